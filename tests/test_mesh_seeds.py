"""The meshes and initial conditions both arms use are the reference's.

- The reference's seed files (mesh_seeds/*.dat, parsed into
  tests/golden/mesh_seeds.npz by tests/golden/make_mesh_seeds.py) hold the
  level-0 vertex coordinates and face centres; the library's seeds
  (lpm_gb300/csrc/mesh.cpp) reproduce them bit for bit.
- The oracle's restatement of PolyMesh2d::tree_init with the reference's
  edge-based dividers (oracle/lpm_oracle_mesh.cpp), grown from those seeds,
  equals the library's mesh bit for bit: vertices, face centres, areas, masks
  and face vertex lists.
- The oracle's restated initial conditions equal the library's.
- Known answers of the reference: total area 4 pi on the unit sphere and
  (2 r)^2 on the square (tests/lpm_geometry_tests.cpp:133-227 checks the seed
  areas), the tree-level counts (src/mesh/lpm_mesh_seed.cpp:306-371).
"""
import math
from pathlib import Path

import numpy as np
import pytest

import lpm_oracle as O
from lpm_gb300 import core

REF_SEEDS = Path("/root/reference/mesh_seeds")
KINDS = [(O.MESH_ICOS_TRI, "icos", 1.0), (O.MESH_CUBED_SPHERE, "cubed", 1.0),
         (O.MESH_QUAD_RECT, "quad", 1.0), (O.MESH_QUAD_RECT, "quad", 4.0)]


@pytest.mark.parametrize("kind,name,radius", KINDS)
def test_library_seed_equals_reference_seed_file(kind, name, radius):
    crds, _, fverts, _ = O.seed(kind)
    nv0 = crds.shape[0] - fverts.shape[0]
    vx, fx, fa, fm = core.build_mesh(kind, 0, radius)
    assert np.array_equal(vx, crds[:nv0] * radius)
    assert np.array_equal(fx, crds[nv0:] * radius)
    assert np.array_equal(core.mesh_face_vertices(kind, 0), fverts)
    assert not fm.any()


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("kind,name,radius", KINDS)
def test_oracle_mesh_equals_library_mesh(kind, name, radius, level):
    vx, fx, fa, fm, fv = O.mesh_build(kind, level, radius)
    lv, lf, la, lm = core.build_mesh(kind, level, radius)
    assert np.array_equal(vx, lv) and np.array_equal(fx, lf)
    assert np.array_equal(fa, la) and np.array_equal(fm, lm)
    assert np.array_equal(fv, core.mesh_face_vertices(kind, level))
    nv, nf = O.mesh_sizes(kind, level)
    assert vx.shape[0] == nv and fx.shape[0] == nf
    leaf = fm == 0
    nleaf = {O.MESH_ICOS_TRI: 20, O.MESH_CUBED_SPHERE: 6, O.MESH_QUAD_RECT: 4}[kind] * 4 ** level
    assert leaf.sum() == nleaf and not fa[~leaf].any()
    if kind == O.MESH_QUAD_RECT:
        assert abs(fa.sum() - (2 * radius) ** 2) < 1e-12 * radius ** 2
    else:
        assert abs(fa.sum() - 4 * math.pi) < 1e-12
        assert np.abs(np.linalg.norm(vx, axis=1) - 1).max() < 4e-16


def test_oracle_initial_conditions_equal_library():
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 4)
    w = 2 * math.pi / 12.5
    cases = [(O.IC_SOLID_BODY, ()),
             (O.IC_GAUSSIAN_SPHERE, (4 * math.pi, 4.0, 0.0, 0.05 * math.pi, 0.0, 2 * math.pi)),
             (O.IC_RH54, (w, -w)),
             (O.IC_MULTI_GAUSSIAN, (2, 3.0, 2.0, 0.1, 0.3, 6.0, 5.0, 1.0, -0.5))]
    for kind, prm in cases:
        assert np.array_equal(O.ic_eval(kind, prm, fx), core.eval_ic(kind, prm, fx))
    qv, qf, qa, qm = O.mesh(O.MESH_QUAD_RECT, 4, 4.0)
    prm = (2.0, 1.0, -2.0, 0.0, -2.0, 1.0, 2.0, 0.0)
    z = O.ic_eval(O.IC_DIPOLE_PAIR, prm, qf)
    assert np.array_equal(z, core.eval_ic(core.IC_DIPOLE_PAIR, prm, qf)) and np.abs(z).max() > 1
    with pytest.raises(ValueError):
        O.ic_eval(O.IC_DIPOLE_PAIR, prm[:3], qf)


@pytest.mark.skipif(not REF_SEEDS.is_dir(), reason="the reference's seed files are not here")
def test_seed_fixture_is_the_reference_files():
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "make_mesh_seeds", Path(__file__).parent / "golden" / "make_mesh_seeds.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    with np.load(Path(__file__).parent / "golden" / "mesh_seeds.npz") as z:
        for name, (fname, ndim, nv, nf, ne, nfv) in mk.SEEDS.items():
            parsed = mk.parse(REF_SEEDS / fname, ndim, nv, nf, ne, nfv)
            for arr, tag in zip(parsed, ("crds", "edges", "faceverts", "faceedges")):
                assert np.array_equal(arr, z[f"{name}_{tag}"]), (name, tag)

"""Host-side checks that need no GPU: the C ABI library loads and exports every
symbol the header declares, meshes have the reference's sizes and geometry,
initial conditions follow the reference gallery."""
import math
import re
from pathlib import Path

import numpy as np
import pytest

from lpm_gb300 import core

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "lpm_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lpm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = core.lib()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(core.EXPORTS) == names


def test_no_gpu_is_reported_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    L = core.lib()
    assert L.lpm_device_count() == 0
    with pytest.raises(core.LpmError) as e:
        core.Context(0)
    assert e.value.code == core.LPM_ERR_CUDA


def test_one_call_argument_checks():
    """The one-call forms reject bad arguments before touching a device."""
    L = core.lib()
    c = core.Crd3(None, 0, 3, 1)
    for fn in (L.lpm_bve_direct_sum, L.lpm_plane_direct_sum):
        assert fn(c, c, None, None, None, 0, 0, 0.0, 0, core.FP64, None, 3, 1, None, None) \
            == core.LPM_ERR_ARG  # want out of range
        assert fn(c, c, None, None, None, 0, 0, -1.0, 1, core.FP64, None, 3, 1, None, None) \
            == core.LPM_ERR_ARG  # negative eps
        d = core.Crd3(None, 5, 3, 1)
        assert fn(d, c, None, None, None, 0, 1, 0.0, 1, core.FP64, None, 3, 1, None, None) \
            == core.LPM_ERR_ARG  # collocated with a different target view
    assert L.lpm_one_call_release() == core.LPM_OK  # nothing cached: a no-op
    v = core.View(None, 0, 0)
    assert L.lpm_ensemble_run(None, -1, v, None, v, v, None, v, None) == core.LPM_ERR_ARG
    assert L.lpm_ensemble_run(None, 0, v, None, v, v, None, v, None) == core.LPM_OK


@pytest.mark.parametrize("kind,level,nv,nf,nleaf", [
    (core.MESH_ICOS_TRI, 4, 2562, 6820, 5120),
    (core.MESH_ICOS_TRI, 7, 163842, 436900, 327680),
    (core.MESH_CUBED_SPHERE, 4, 1538, 2046, 1536),
    (core.MESH_QUAD_RECT, 4, 33 * 33, 1364, 1024),
])
def test_mesh_sizes_match_reference_formulas(kind, level, nv, nf, nleaf):
    assert core.mesh_sizes(kind, level) == (nv, nf)
    if level <= 4:
        vx, fx, fa, fm = core.build_mesh(kind, level, 1.0)
        assert vx.shape[0] == nv and fx.shape[0] == nf and int((fm == 0).sum()) == nleaf
        assert np.all(fa[fm == 1] == 0) and np.all(fa[fm == 0] > 0)


def test_quad_level9_is_1024_squared():
    nv, nf = core.mesh_sizes(core.MESH_QUAD_RECT, 9)
    assert nv == 1025 * 1025
    assert nf == sum(4 * 4 ** i for i in range(10))


@pytest.mark.parametrize("kind", [core.MESH_ICOS_TRI, core.MESH_CUBED_SPHERE])
def test_sphere_mesh_geometry(kind):
    vx, fx, fa, fm = core.build_mesh(kind, 3, 1.0)
    leaf = fm == 0
    assert math.isclose(fa[leaf].sum(), 4 * math.pi, rel_tol=1e-12)
    assert np.abs(np.linalg.norm(vx, axis=1) - 1).max() < 1e-15
    assert np.abs(np.linalg.norm(fx, axis=1) - 1).max() < 1e-15


def test_cubed_sphere_seed_face_area():
    # polygon_area of the cube face around (1,0,0) is 2 pi / 3
    # (tests/lpm_geometry_tests.cpp:218-224)
    vx, fx, fa, fm = core.build_mesh(core.MESH_CUBED_SPHERE, 0, 1.0)
    assert np.allclose(fa, 2 * math.pi / 3, rtol=0, atol=1e-14)
    assert np.allclose(np.abs(fx).max(1), 1.0)


def test_quad_rect_geometry():
    vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, 3, 4.0)
    leaf = fm == 0
    assert math.isclose(fa[leaf].sum(), 64.0, rel_tol=1e-14)
    assert np.allclose(fa[leaf], (8.0 / 16) ** 2)
    assert vx.min() == -4.0 and vx.max() == 4.0


def test_children_follow_parents_level_by_level():
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, 2, 1.0)
    # 20 seed faces, then 80 level-1, then 320 level-2 slots; only the last are leaves
    assert np.all(fm[:100] == 1) and np.all(fm[100:] == 0)
    # each parent's four children have areas summing to the parent's original area
    vx1, fx1, fa1, fm1 = core.build_mesh(core.MESH_ICOS_TRI, 1, 1.0)
    assert np.allclose(fa1[20:].reshape(20, 4).sum(1), 4 * math.pi / 20, rtol=1e-12)


def test_initial_conditions():
    x = np.array([[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0], [0.6, 0, 0.8]])
    sb = core.eval_ic(core.IC_SOLID_BODY, (), x)
    assert np.allclose(sb, 4 * math.pi * x[:, 2])
    g = core.eval_ic(core.IC_GAUSSIAN_SPHERE, (4 * math.pi, 4.0, 0.0, math.pi / 20, 0.0, 2 * math.pi), x)
    c = np.array([math.cos(math.pi / 20), 0, math.sin(math.pi / 20)])
    assert np.allclose(g, 4 * math.pi * np.exp(-16 * (1 - x @ c)) + 4 * math.pi * x[:, 2])
    w = 2 * math.pi / 12.5
    rh = core.eval_ic(core.IC_RH54, (w, -w), x)
    lon = np.mod(np.arctan2(x[:, 1], x[:, 0]), 2 * math.pi)
    z = x[:, 2]
    assert np.allclose(rh, 2 * w * z - 30 * w * np.cos(4 * lon) * z * (z * z - 1) ** 2)
    # Lamb dipole: zero outside the radius, odd in y about the centre line
    p = np.array([[-2.0, 0.5], [-2.0, -0.5], [0.0, 0.0], [-2.0, 0.0]])
    d = core.eval_ic(core.IC_DIPOLE_PAIR, (2.0, 1.0, -2.0, 0.0, -2.0, 1.0, 2.0, 0.0), p)
    assert d[2] == 0 and d[3] == 0 and math.isclose(d[0], -d[1])


def test_ic_argument_errors():
    with pytest.raises(core.LpmError):
        core.eval_ic(core.IC_GAUSSIAN_SPHERE, (1.0,), np.zeros((2, 3)))
    with pytest.raises(core.LpmError):
        core.eval_ic(99, (), np.zeros((2, 3)))
    with pytest.raises(core.LpmError):
        core.mesh_sizes(99, 2)

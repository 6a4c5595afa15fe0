"""Generates the golden fixtures under tests/golden/ with the FP64 oracle.

    python tests/golden/make_golden.py

The reference itself cannot be built here (it needs Kokkos and friends), so
the fixtures hold the oracle's outputs on small seeded inputs: the
reference's own meshes (grown by the oracle's restatement of tree_init from
the reference's seed files, tests/golden/mesh_seeds.npz) and initial
conditions restated by the oracle, so no product code is involved.  They
freeze the oracle (checked on CPU on every platform) and give the CUDA path a
fixed target independent of the live oracle.
"""
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import lpm_oracle as O  # noqa: E402

OMEGA = 2 * math.pi


def bve_case():
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    w = OMEGA / 12.5
    fz = O.ic_eval(O.IC_RH54, (w, -w), fx)
    fz = fz + 0.25 * np.random.default_rng(11).standard_normal(fz.shape)
    vz = O.ic_eval(O.IC_RH54, (w, -w), vx)
    vpsi, vu = O.bve_vertex_solve(vx, fx, fz, fa, fm)
    fpsi, fu = O.bve_face_solve(fx, fz, fa, fm)
    s = O.BVEState(vx, vz, vu, fx, fz, fu, fa, fm)
    for _ in range(2):
        s.step(0.01, OMEGA)
    np.savez_compressed(HERE / "bve_icos_l2.npz", vx=vx, fx=fx, fa=fa, fm=fm, vz=vz, fz=fz,
                        vpsi=vpsi, vu=vu, fpsi=fpsi, fu=fu, step_vx=s.vx, step_fx=s.fx,
                        step_vz=s.vzeta, step_fz=s.fzeta, step_vu=s.vvel, step_fu=s.fvel,
                        dt=0.01, nsteps=2)


def ic2d_sphere_case():
    vx, fx, fa, fm = O.mesh(O.MESH_CUBED_SPHERE, 2, 1.0)
    prm = (4 * math.pi, 4.0, 0.0, math.pi / 20, 0.0, 0.0)
    fz = O.ic_eval(O.IC_GAUSSIAN_SPHERE, prm, fx)
    out = {}
    for eps in (0.0, 0.05):
        up, pp = O.ic2d_passive_sums(vx, fx, fz, fa, fm, eps)
        ua, pa = O.ic2d_active_sums(fx, fz, fa, fm, eps)
        tag = "e0" if eps == 0 else "e5"
        out.update({f"up_{tag}": up, f"pp_{tag}": pp, f"ua_{tag}": ua, f"pa_{tag}": pa})
    np.savez_compressed(HERE / "ic2d_cubed_l2.npz", vx=vx, fx=fx, fa=fa, fm=fm, fz=fz, **out)


def ic2d_plane_case():
    vx, fx, fa, fm = O.mesh(O.MESH_QUAD_RECT, 3, 4.0)
    prm = (2.0, 1.0, -2.0, 0.0, -2.0, 1.0, 2.0, 0.0)
    fz = O.ic_eval(O.IC_DIPOLE_PAIR, prm, fx)
    vz = O.ic_eval(O.IC_DIPOLE_PAIR, prm, vx)
    up, pp = O.ic2d_passive_sums(vx, fx, fz, fa, fm, 0.02)
    ua, pa = O.ic2d_active_sums(fx, fz, fa, fm, 0.02)
    s = O.IC2DState(vx, vz, fx, fz, fa, fm, 0.02, 0.0)
    s.init_direct_sums()
    for _ in range(2):
        s.step(0.01)
    np.savez_compressed(HERE / "ic2d_quad_l3.npz", vx=vx, fx=fx, fa=fa, fm=fm, vz=vz, fz=fz,
                        up=up, pp=pp, ua=ua, pa=pa, step_vx=s.vx, step_fx=s.fx,
                        step_fz=s.fzeta, step_fu=s.fvel, step_fpsi=s.fpsi, eps=0.02, dt=0.01,
                        nsteps=2)


if __name__ == "__main__":
    O.set_threads(1)
    bve_case()
    ic2d_sphere_case()
    ic2d_plane_case()
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)

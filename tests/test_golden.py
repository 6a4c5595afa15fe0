"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the mesh generator and the oracle reproduce the fixtures on this
platform.  GPU: the CUDA path reproduces them (FP64 1e-12, FP32C 2e-6).
"""
import math
from pathlib import Path

import numpy as np
import pytest

from lpm_gb300 import core

G = Path(__file__).resolve().parent / "golden"
OMEGA = 2 * math.pi


def load(name):
    return dict(np.load(G / name))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb)
    a, b = a[fb], b[fb]
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_mesh_and_ics_reproduce_fixtures():
    d = load("bve_icos_l2.npz")
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, 2, 1.0)
    assert rel(vx, d["vx"]) < 1e-15 and rel(fx, d["fx"]) < 1e-15
    assert rel(fa, d["fa"]) < 1e-13 and np.array_equal(fm, d["fm"])
    q = load("ic2d_quad_l3.npz")
    vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, 3, 4.0)
    assert np.array_equal(vx, q["vx"]) and np.array_equal(fx, q["fx"])
    fz = core.eval_ic(core.IC_DIPOLE_PAIR, (2.0, 1.0, -2.0, 0.0, -2.0, 1.0, 2.0, 0.0), fx)
    assert rel(fz, q["fz"]) < 1e-13


def test_oracle_reproduces_fixtures(oracle):
    d = load("bve_icos_l2.npz")
    vpsi, vu = oracle.bve_vertex_solve(d["vx"], d["fx"], d["fz"], d["fa"], d["fm"])
    fpsi, fu = oracle.bve_face_solve(d["fx"], d["fz"], d["fa"], d["fm"])
    for got, want in ((vpsi, "vpsi"), (vu, "vu"), (fpsi, "fpsi"), (fu, "fu")):
        assert rel(got, d[want]) < 1e-13, want
    s = oracle.BVEState(d["vx"], d["vz"], d["vu"], d["fx"], d["fz"], d["fu"], d["fa"], d["fm"])
    for _ in range(int(d["nsteps"])):
        s.step(float(d["dt"]), OMEGA)
    assert rel(s.fx, d["step_fx"]) < 1e-13 and rel(s.fvel, d["step_fu"]) < 1e-13
    c = load("ic2d_cubed_l2.npz")
    for eps, tag in ((0.0, "e0"), (0.05, "e5")):
        up, pp = oracle.ic2d_passive_sums(c["vx"], c["fx"], c["fz"], c["fa"], c["fm"], eps)
        ua, pa = oracle.ic2d_active_sums(c["fx"], c["fz"], c["fa"], c["fm"], eps)
        assert rel(up, c[f"up_{tag}"]) < 1e-13 and rel(pp, c[f"pp_{tag}"]) < 1e-13
        assert rel(ua, c[f"ua_{tag}"]) < 1e-13 and rel(pa, c[f"pa_{tag}"]) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [core.FP64, core.FP32C])
def test_cuda_path_reproduces_fixtures(gpu_ctx, precision):
    import torch

    from lpm_gb300 import functors as F

    ctx = gpu_ctx
    ctx.set_precision(precision)
    tol = 1e-12 if precision == core.FP64 else 2e-6
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    d = load("bve_icos_l2.npz")
    leaf = d["fm"] == 0
    vu = torch.zeros(d["vx"].shape[0], 3, dtype=torch.float64, device="cuda")
    vp = torch.zeros(d["vx"].shape[0], dtype=torch.float64, device="cuda")
    fu = torch.zeros(d["fx"].shape[0], 3, dtype=torch.float64, device="cuda")
    fp = torch.zeros(d["fx"].shape[0], dtype=torch.float64, device="cuda")
    F.bve_vertex_solve(ctx, vp, vu, dev(d["vx"]), dev(d["fx"]), dev(d["fz"]), dev(d["fa"]),
                       dev(d["fm"]))
    F.bve_face_solve(ctx, fp, fu, dev(d["fx"]), dev(d["fz"]), dev(d["fa"]), dev(d["fm"]))
    ctx.synchronize()
    assert rel(vu.cpu(), d["vu"]) < tol and rel(vp.cpu(), d["vpsi"]) < tol
    assert rel(fu.cpu().numpy()[leaf], d["fu"][leaf]) < tol
    assert rel(fp.cpu().numpy()[leaf], d["fpsi"][leaf]) < tol
    q = load("ic2d_quad_l3.npz")
    qu = torch.zeros(q["fx"].shape[0], 2, dtype=torch.float64, device="cuda")
    qp = torch.zeros(q["fx"].shape[0], dtype=torch.float64, device="cuda")
    F.ic2d_active_sums(ctx, qu, qp, dev(q["fx"]), dev(q["fz"]), dev(q["fa"]), dev(q["fm"]),
                       float(q["eps"]))
    ctx.synchronize()
    ql = q["fm"] == 0
    assert rel(qu.cpu().numpy()[ql], q["ua"][ql]) < tol
    assert rel(qp.cpu().numpy()[ql], q["pa"][ql]) < tol

"""Device steppers (BVERK4, Incompressible2DRK2) vs the oracle's steppers."""
import math

import numpy as np
import pytest
import torch

from lpm_gb300 import core
from lpm_gb300.bve import BVERK4, BVESphere, gaussian_params, rossby_haurwitz_params
from lpm_gb300.ic2d import Incompressible2D, Incompressible2DRK2, colliding_dipoles_params

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi


def rel(a, b, sel=slice(None)):
    a = np.asarray(a, np.float64)[sel]
    b = np.asarray(b, np.float64)[sel]
    den = np.abs(b).max()
    return np.abs(a - b).max() / (den if den > 0 else 1.0)


def oracle_bve(oracle, sph):
    return oracle.BVEState(sph.vert_x.cpu().numpy(), sph.rel_vort_verts.cpu().numpy(),
                           sph.velocity_verts.cpu().numpy(), sph.face_x.cpu().numpy(),
                           sph.rel_vort_faces.cpu().numpy(), sph.velocity_faces.cpu().numpy(),
                           sph.host_face_area, sph.host_face_mask)


@pytest.mark.parametrize("eps", [0.0, 0.02])
@pytest.mark.parametrize("flags", [0, core.STEP_FIX_FACEVORT3 | core.STEP_REPROJECT,
                                   core.STEP_SKIP_MASKED_TARGETS, core.STEP_NO_GRAPH])
def test_bve_rk4_fp64(gpu_ctx, oracle, eps, flags):
    ctx = gpu_ctx
    ctx.set_precision(core.FP64)
    sph = BVESphere(3, ctx=ctx)
    sph.init_vorticity(core.IC_RH54, rossby_haurwitz_params())
    sph.init_velocity()
    if eps:
        # with smoothing the entry velocity comes from the eps kernel
        from lpm_gb300 import functors as F
        F.ic2d_passive_sums(ctx, sph.velocity_verts, None, sph.vert_x, sph.face_x,
                            sph.rel_vort_faces, sph.face_area, sph.face_mask, eps)
        F.ic2d_active_sums(ctx, sph.velocity_faces, None, sph.face_x, sph.rel_vort_faces,
                           sph.face_area, sph.face_mask, eps, self_rule=1)
    ctx.synchronize()
    ref = oracle_bve(oracle, sph)
    st = BVERK4(0.01, sph, precision=core.FP64, eps=eps, flags=flags)
    for _ in range(3):
        st.advance_timestep(sph)
        ref.step(0.01, OMEGA, eps, bool(flags & core.STEP_FIX_FACEVORT3),
                 bool(flags & core.STEP_REPROJECT))
    ctx.synchronize()
    leaf = sph.host_face_mask == 0
    sel = leaf if flags & core.STEP_SKIP_MASKED_TARGETS else slice(None)
    assert rel(sph.vert_x.cpu(), ref.vx) < 1e-12
    assert rel(sph.face_x.cpu(), ref.fx, sel) < 1e-12
    assert rel(sph.rel_vort_faces.cpu(), ref.fzeta, sel) < 1e-12
    assert rel(sph.rel_vort_verts.cpu(), ref.vzeta) < 1e-12
    assert rel(sph.velocity_verts.cpu(), ref.vvel) < 1e-12
    assert rel(sph.velocity_faces.cpu(), ref.fvel, sel) < 1e-12


def test_bve_rk4_fp32c(gpu_ctx, oracle):
    ctx = gpu_ctx
    ctx.set_precision(core.FP64)
    sph = BVESphere(4, ctx=ctx)
    sph.init_vorticity(core.IC_GAUSSIAN_SPHERE, gaussian_params(background_Omega=OMEGA))
    sph.init_velocity()
    ctx.synchronize()
    ref = oracle_bve(oracle, sph)
    st = BVERK4(0.005, sph, precision=core.FP32C, flags=core.STEP_SKIP_MASKED_TARGETS)
    for _ in range(2):
        st.advance_timestep(sph)
        ref.step(0.005, OMEGA)
    ctx.synchronize()
    leaf = sph.host_face_mask == 0
    assert rel(sph.velocity_verts.cpu(), ref.vvel) < 2e-6
    assert rel(sph.velocity_faces.cpu(), ref.fvel, leaf) < 2e-6
    assert rel(sph.face_x.cpu(), ref.fx, leaf) < 1e-9
    assert rel(sph.rel_vort_faces.cpu(), ref.fzeta, leaf) < 1e-8


def test_graph_replay_equals_direct(gpu_ctx):
    ctx = gpu_ctx
    out = []
    for flags in (0, core.STEP_NO_GRAPH):
        sph = BVESphere(3, ctx=ctx)
        sph.init_vorticity(core.IC_RH54, rossby_haurwitz_params())
        ctx.set_precision(core.FP32C)
        sph.init_velocity()
        st = BVERK4(0.01, sph, precision=core.FP32C, flags=flags)
        for _ in range(3):
            st.advance_timestep(sph)
        ctx.synchronize()
        out.append((sph.face_x.clone(), sph.velocity_faces.clone()))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])


@pytest.mark.parametrize("precision", [core.FP64, core.FP32C])
@pytest.mark.parametrize("case", ["sphere0", "sphere_eps", "plane"])
def test_ic2d_rk2(gpu_ctx, oracle, precision, case):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    if case == "plane":
        ic = Incompressible2D(core.MESH_QUAD_RECT, 3, radius=4.0, eps=0.02, ctx=ctx)
        ic.init_vorticity(core.IC_DIPOLE_PAIR, colliding_dipoles_params())
    else:
        eps = 0.0 if case == "sphere0" else 0.05
        ic = Incompressible2D(core.MESH_CUBED_SPHERE, 3, eps=eps, ctx=ctx)
        ic.init_vorticity(core.IC_GAUSSIAN_SPHERE, (4 * math.pi, 4.0, 0.0, math.pi / 20, 0, 0))
    ref = oracle.IC2DState(ic.vert_x.cpu().numpy(), ic.rel_vort_passive.cpu().numpy(),
                           ic.face_x.cpu().numpy(), ic.rel_vort_active.cpu().numpy(),
                           ic.face_area.cpu().numpy(), ic.host_face_mask, ic.eps, ic.cor_param)
    ref.init_direct_sums()
    ic.init_direct_sums()
    solver = Incompressible2DRK2(0.01, ic, precision=precision)
    for _ in range(3):
        ic.advance_timestep(solver)
        ref.step(0.01)
    ctx.synchronize()
    leaf = ic.host_face_mask == 0
    if precision == core.FP64:
        tol, sel, tx = 1e-12, slice(None), 1e-12
    else:
        tol, sel, tx = 2e-6, leaf, 1e-8
    assert rel(ic.face_x.cpu(), ref.fx, sel) < tx
    assert rel(ic.vert_x.cpu(), ref.vx) < tx
    assert rel(ic.velocity_active.cpu(), ref.fvel, sel) < tol
    assert rel(ic.velocity_passive.cpu(), ref.vvel) < tol
    assert rel(ic.stream_fn_active.cpu(), ref.fpsi, sel) < tol
    assert rel(ic.stream_fn_passive.cpu(), ref.vpsi) < tol
    assert rel(ic.rel_vort_active.cpu(), ref.fzeta, sel) < tx
    assert abs(ic.t - 0.03) < 1e-15

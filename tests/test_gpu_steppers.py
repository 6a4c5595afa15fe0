"""Device steppers (BVERK4, Incompressible2DRK2) vs the oracle's steppers.

FP64 (the reference's arithmetic) is compared with the reference-form oracle
to 1e-12 on vertices and leaf faces.  Divided parent slots are left out after
the first stage: in the reference's arithmetic a parent whose centre
coincides with its central child's gets a near-singular (or non-finite)
velocity, so its later positions depend on round-off in any implementation.
The chord modes (FP64_CHORD, FP32C) are compared with the chord-form oracle.
"""
import math

import numpy as np
import pytest
import torch

from lpm_gb300 import core
from lpm_gb300 import functors as F
from lpm_gb300.bve import BVERK4, BVESphere, gaussian_params, rossby_haurwitz_params
from lpm_gb300.ic2d import Incompressible2D, Incompressible2DRK2, colliding_dipoles_params

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi
# (velocity / stream function, positions); FP32C positions carry the ~1e-7
# velocity error times dt |u| per step
TOLS = {core.FP64: (1e-12, 1e-12), core.FP64_CHORD: (1e-11, 1e-12), core.FP32C: (2e-6, 1e-7)}


def rel(a, b, sel=slice(None)):
    """max|a-b| / max|b| over finite entries; non-finite entries must match."""
    a = np.asarray(a, np.float64)[sel]
    b = np.asarray(b, np.float64)[sel]
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), "non-finite entries differ"
    a, b = a[fb], b[fb]
    if b.size == 0:
        return 0.0
    den = np.abs(b).max()
    return np.abs(a - b).max() / (den if den > 0 else 1.0)


def oracle_bve(oracle, sph):
    return oracle.BVEState(sph.vert_x.cpu().numpy(), sph.rel_vort_verts.cpu().numpy(),
                           sph.velocity_verts.cpu().numpy(), sph.face_x.cpu().numpy(),
                           sph.rel_vort_faces.cpu().numpy(), sph.velocity_faces.cpu().numpy(),
                           sph.host_face_area, sph.host_face_mask)


def entry_velocity(ctx, sph, eps):
    if eps == 0:
        sph.init_velocity()
    else:
        F.ic2d_passive_sums(ctx, sph.velocity_verts, None, sph.vert_x, sph.face_x,
                            sph.rel_vort_faces, sph.face_area, sph.face_mask, eps)
        F.ic2d_active_sums(ctx, sph.velocity_faces, None, sph.face_x, sph.rel_vort_faces,
                           sph.face_area, sph.face_mask, eps, self_rule=1)
    ctx.synchronize()


@pytest.mark.parametrize("eps", [0.0, 0.02])
@pytest.mark.parametrize("flags", [0, core.STEP_FIX_FACEVORT3 | core.STEP_REPROJECT,
                                   core.STEP_SKIP_MASKED_TARGETS, core.STEP_NO_GRAPH])
def test_bve_rk4_fp64(gpu_ctx, oracle, eps, flags):
    ctx = gpu_ctx
    ctx.set_precision(core.FP64)
    sph = BVESphere(3, ctx=ctx)
    sph.init_vorticity(core.IC_RH54, rossby_haurwitz_params())
    entry_velocity(ctx, sph, eps)
    ref = oracle_bve(oracle, sph)
    st = BVERK4(0.01, sph, precision=core.FP64, eps=eps, flags=flags)
    for _ in range(3):
        st.advance_timestep(sph)
        ref.step(0.01, OMEGA, eps, bool(flags & core.STEP_FIX_FACEVORT3),
                 bool(flags & core.STEP_REPROJECT))
    ctx.synchronize()
    leaf = sph.host_face_mask == 0
    assert rel(sph.vert_x.cpu(), ref.vx) < 1e-12
    assert rel(sph.rel_vort_verts.cpu(), ref.vzeta) < 1e-12
    assert rel(sph.velocity_verts.cpu(), ref.vvel) < 1e-12
    assert rel(sph.face_x.cpu(), ref.fx, leaf) < 1e-12
    assert rel(sph.rel_vort_faces.cpu(), ref.fzeta, leaf) < 1e-12
    assert rel(sph.velocity_faces.cpu(), ref.fvel, leaf) < 1e-12
    if flags & core.STEP_SKIP_MASKED_TARGETS:
        # parent slots are neither evaluated nor moved
        par = ~leaf
        assert np.array_equal(sph.face_x.cpu().numpy()[par], sph.host_face_x[par])


@pytest.mark.parametrize("precision", [core.FP64_CHORD, core.FP32C])
@pytest.mark.parametrize("reproject", [False, True])
def test_bve_rk4_chord(gpu_ctx, oracle, precision, reproject):
    ctx = gpu_ctx
    ctx.set_precision(core.FP64)
    sph = BVESphere(4, ctx=ctx)
    sph.init_vorticity(core.IC_GAUSSIAN_SPHERE, gaussian_params(background_Omega=OMEGA))
    eps = 0.01
    entry_velocity(ctx, sph, eps)
    ref = oracle_bve(oracle, sph)
    flags = core.STEP_SKIP_MASKED_TARGETS | (core.STEP_REPROJECT if reproject else 0)
    st = BVERK4(0.005, sph, precision=precision, eps=eps, flags=flags)
    with oracle.chord_form():
        for _ in range(2):
            st.advance_timestep(sph)
            ref.step(0.005, OMEGA, eps, reproject=reproject)
    ctx.synchronize()
    tol, tx = TOLS[precision]
    leaf = sph.host_face_mask == 0
    assert rel(sph.velocity_verts.cpu(), ref.vvel) < tol
    assert rel(sph.velocity_faces.cpu(), ref.fvel, leaf) < tol
    assert rel(sph.face_x.cpu(), ref.fx, leaf) < tx
    assert rel(sph.rel_vort_faces.cpu(), ref.fzeta, leaf) < tx * 100


def test_graph_replay_equals_direct(gpu_ctx):
    ctx = gpu_ctx
    out = []
    for flags in (0, core.STEP_NO_GRAPH, core.STEP_TIME_NBODY):
        sph = BVESphere(3, ctx=ctx)
        sph.init_vorticity(core.IC_RH54, rossby_haurwitz_params())
        ctx.set_precision(core.FP32C)
        sph.init_velocity()
        st = BVERK4(0.01, sph, precision=core.FP32C, flags=flags)
        for _ in range(3):
            st.advance_timestep(sph)
        ctx.synchronize()
        if flags == core.STEP_TIME_NBODY:
            ms, n = st.nbody_time()
            assert n == 12 and ms > 0
        out.append((sph.face_x.clone(), sph.velocity_faces.clone()))
    for o in out[1:]:
        assert torch.equal(out[0][0], o[0]) and torch.equal(out[0][1], o[1])


def test_stepper_reports_its_kernel_shape(gpu_ctx):
    """lpm_bve_rk4_kernel_shape: an error before the first step; afterwards
    the shape fixed through lpm_context_set_kernel_shape (index 3: 256
    threads x 2 targets, 5 CTAs per SM), or one of the six autotuned ones."""
    ctx = gpu_ctx
    table = {(256, 4, 3), (256, 4, 4), (128, 8, 4), (256, 2, 5), (128, 8, 3), (256, 4, 2)}
    for fixed in (3, -1):
        ctx.set_kernel_shape(fixed)
        try:
            sph = BVESphere(4, ctx=ctx)
            sph.init_vorticity(core.IC_RH54, rossby_haurwitz_params())
            ctx.set_precision(core.FP32C)
            sph.init_velocity()
            st = BVERK4(0.01, sph, precision=core.FP32C)
            with pytest.raises(core.LpmError):
                st.kernel_shape()
            st.advance_timestep(sph)
            ctx.synchronize()
            shape = st.kernel_shape()
            assert shape == (256, 2, 5) if fixed == 3 else shape in table
            st.close()
        finally:
            ctx.set_kernel_shape(-1)


@pytest.mark.parametrize("precision", [core.FP64, core.FP64_CHORD, core.FP32C])
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
    oracle.set_sphere_form(precision != core.FP64)
    try:
        ref.init_direct_sums()
        ic.init_direct_sums()
        solver = Incompressible2DRK2(0.01, ic, precision=precision)
        for _ in range(3):
            ic.advance_timestep(solver)
            ref.step(0.01)
    finally:
        oracle.set_sphere_form(False)
    ctx.synchronize()
    leaf = ic.host_face_mask == 0
    tol, tx = TOLS[precision]
    assert rel(ic.face_x.cpu(), ref.fx, leaf) < tx
    assert rel(ic.vert_x.cpu(), ref.vx) < tx
    assert rel(ic.velocity_active.cpu(), ref.fvel, leaf) < tol
    assert rel(ic.velocity_passive.cpu(), ref.vvel) < tol
    assert rel(ic.stream_fn_active.cpu(), ref.fpsi, leaf) < tol
    assert rel(ic.stream_fn_passive.cpu(), ref.vpsi) < tol
    assert rel(ic.rel_vort_active.cpu(), ref.fzeta, leaf) < tx * 100
    assert abs(ic.t - 0.03) < 1e-15


def test_reference_form_breaks_off_sphere(gpu_ctx, oracle):
    """At RK stage positions (off the unit sphere by O(dt^2 |u|^2)) the
    reference's 1 - x.y + eps^2 goes non-positive for near neighbours on fine
    meshes; the chord form does not.  Level 6, Gaussian + 2 Omega z, dt 0.005."""
    ctx = gpu_ctx
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, 6, 1.0)
    prm = (4 * math.pi, 4.0, 0.0, 0.05 * math.pi, 0.0, OMEGA)
    fz = core.eval_ic(core.IC_GAUSSIAN_SPHERE, prm, fx)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = torch.zeros(fx.shape[0], 3, dtype=torch.float64, device="cuda")
    ctx.set_precision(core.FP64_CHORD)
    F.ic2d_active_sums(ctx, u, None, dev(fx), dev(fz), dev(fa), dev(fm), 0.01, self_rule=1)
    ctx.synchronize()
    xw = fx + 0.5 * 0.005 * u.cpu().numpy()  # RK4 stage-2 positions
    leaf = np.nonzero(fm == 0)[0]
    nonpositive = 0
    for i in leaf[:: len(leaf) // 64][:64]:
        arg = 1 - xw[leaf] @ xw[i] + 0.01 ** 2
        arg[leaf == i] = 1.0
        nonpositive += int((arg <= 0).sum())
        chord = 0.5 * ((xw[leaf] - xw[i]) ** 2).sum(1) + 0.01 ** 2
        assert (chord > 0).all()
    assert nonpositive > 0

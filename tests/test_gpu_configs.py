"""The CUDA path against the oracle at the benchmark configurations' sizes.

Inputs come from the oracle (the reference's meshes grown from its seed
files and its initial conditions), so the oracle's side of every comparison
uses no code of the library.  Where the oracle would take minutes the GPU
result is checked on a seeded sample of targets against all sources.

  C1  icosahedral level 4, Rossby-Haurwitz R = 4 (omega = K = Omega/12.5),
      eps = 0, dt = 0.01, 10 RK4 steps in FP64 with the reference's quirks
      (every face slot evaluated, facevort4, no reprojection): vertices and
      leaf faces within 1e-12 (src/lpm_bve_rk4_impl.hpp:63-167).
  C2  icosahedral level 7, Gaussian vortex + 2 Omega z, eps = 0.01: one
      evaluation of every target; 2,048 seeded targets against the oracle,
      FP64 1e-12, FP32C 1e-6.
  C3  quad level 9 on [-4, 4]^2, colliding dipoles, eps = 0.02: 2,048 seeded
      targets, FP64 1e-12, FP32C 1e-6 (velocity) and 2e-6 (stream function).
  L9  icosahedral level 9 sources (5.2 M) for 4,096 seeded targets, FP64
      1e-12, FP32C 1e-6: the largest index ranges of the suite.
  ic2d_dt_conv  tests/lpm_ic2d_tests.cpp:165-188 on the GPU stepper: cubed
      sphere depth 4, eps = 0, t_f = 0.5, steps {15, 30, 60}, the finest as
      the reference solution, rates > 1.95 in l1, l2 and linf.
  C4  the ensemble (one N-body launch per evaluation for all problems, in
      the kernel form its autotuner chose) against the oracle directly, per
      problem, after one evaluation and two RK4 steps.
"""
import math

import numpy as np
import pytest
import torch

import lpm_oracle as O
from lpm_gb300 import core
from lpm_gb300 import functors as F

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), "non-finite entries differ"
    return np.abs(a[fb] - b[fb]).max() / np.abs(b[fb]).max()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def zeros(*shape):
    return torch.zeros(*shape, dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("precision", [core.FP64, core.FP64_EXACT])
def test_c1_full_run(gpu_ctx, oracle, precision):
    import ctypes as C

    ctx = gpu_ctx
    ctx.set_precision(precision)
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 4)
    w = OMEGA / 12.5
    vz, fz = O.ic_eval(O.IC_RH54, (w, -w), vx), O.ic_eval(O.IC_RH54, (w, -w), fx)
    _, vu = oracle.bve_vertex_solve(vx, fx, fz, fa, fm, want_psi=False)
    _, fu = oracle.bve_face_solve(fx, fz, fa, fm, want_psi=False)
    ref = oracle.BVEState(vx, vz, vu, fx, fz, fu, fa, fm)
    T = {k: dev(v) for k, v in dict(vx=vx, vz=vz, fx=fx, fz=fz, fa=fa, fm=fm).items()}
    T["vu"], T["fu"] = zeros(vx.shape[0], 3), zeros(fx.shape[0], 3)
    F.bve_vertex_velocity(ctx, T["vu"], T["vx"], T["fx"], T["fz"], T["fa"], T["fm"])
    F.bve_face_velocity(ctx, T["fu"], T["fx"], T["fz"], T["fa"], T["fm"])
    h = C.c_void_p()
    core.check(core.lib().lpm_bve_rk4_create(ctx.handle, C.byref(h), vx.shape[0], fx.shape[0],
                                             0.01, OMEGA, 0.0, precision, 0))
    try:
        for _ in range(10):
            core.check(core.lib().lpm_bve_rk4_advance_timestep(
                h, core.view(T["vx"]), core.ptr(T["vz"]), core.view(T["vu"]),
                core.view(T["fx"]), core.ptr(T["fz"]), core.view(T["fu"]), core.ptr(T["fa"]),
                core.ptr(T["fm"])))
            ref.step(0.01, OMEGA)
        ctx.synchronize()
    finally:
        core.lib().lpm_bve_rk4_destroy(h)
    leaf = fm == 0
    g = {k: v.cpu().numpy() for k, v in T.items()}
    assert rel(g["vx"], ref.vx) < 1e-12
    assert rel(g["vz"], ref.vzeta) < 1e-12
    assert rel(g["vu"], ref.vvel) < 1e-12
    assert rel(g["fx"][leaf], ref.fx[leaf]) < 1e-12
    assert rel(g["fz"][leaf], ref.fzeta[leaf]) < 1e-12
    assert rel(g["fu"][leaf], ref.fvel[leaf]) < 1e-12


def sample(n, k, seed, among=None):
    rng = np.random.default_rng(seed)
    pool = np.arange(n) if among is None else np.flatnonzero(among)
    return np.sort(rng.choice(pool, k, replace=False))


@pytest.mark.parametrize("precision,tol", [(core.FP64, 1e-12), (core.FP32C, 1e-6)])
def test_c2_level7_one_evaluation(gpu_ctx, oracle, precision, tol):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    eps = 0.01
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 7)
    fz = O.ic_eval(O.IC_GAUSSIAN_SPHERE, (4 * math.pi, 4.0, 0.0, 0.05 * math.pi, 0.0, OMEGA), fx)
    T = [dev(a) for a in (vx, fx, fz, fa, fm)]
    vu, fu = zeros(vx.shape[0], 3), zeros(fx.shape[0], 3)
    F.ic2d_passive_sums(ctx, vu, None, T[0], T[1], T[2], T[3], T[4], eps)
    F.ic2d_active_sums(ctx, fu, None, T[1], T[2], T[3], T[4], eps, self_rule=1)
    ctx.synchronize()
    iv = sample(vx.shape[0], 1024, 1)
    jf = sample(fx.shape[0], 1024, 2, fm == 0)
    ru, _ = oracle.ic2d_passive_sums(vx, fx, fz, fa, fm, eps, tgt_idx=iv, want_psi=False)
    rf, _ = oracle.ic2d_active_sums(fx, fz, fa, fm, eps, self_rule=1, tgt_idx=jf)
    got = np.concatenate([vu.cpu().numpy()[iv], fu.cpu().numpy()[jf]])
    assert rel(got, np.concatenate([ru, rf])) < tol


@pytest.mark.parametrize("precision,tol,tolp", [(core.FP64, 1e-12, 1e-12),
                                                (core.FP32C, 1e-6, 2e-6)])
def test_c3_quad9_sample(gpu_ctx, oracle, precision, tol, tolp):
    """With eps > 0 the reference's active sums keep the self pair
    (src/lpm_incompressible2d_kernels.hpp:235), so a face target's sums equal
    the passive sums at its centre: the sample is evaluated that way."""
    ctx = gpu_ctx
    ctx.set_precision(precision)
    eps = 0.02
    vx, fx, fa, fm = O.mesh(O.MESH_QUAD_RECT, 9, 4.0)
    prm = (2.0, 1.0, -2.0, 0.0, -2.0, 1.0, 2.0, 0.0)
    fz = O.ic_eval(O.IC_DIPOLE_PAIR, prm, fx)
    iv = sample(vx.shape[0], 1024, 3)
    jf = sample(fx.shape[0], 1024, 4, fm == 0)
    tx = np.concatenate([vx[iv], fx[jf]])
    u, p = zeros(tx.shape[0], 2), zeros(tx.shape[0])
    F.ic2d_passive_sums(ctx, u, p, dev(tx), dev(fx), dev(fz), dev(fa), dev(fm), eps)
    ctx.synchronize()
    ru, rp = oracle.ic2d_passive_sums(tx, fx, fz, fa, fm, eps)
    ra, rpa = oracle.ic2d_active_sums(fx, fz, fa, fm, eps, tgt_idx=jf)
    assert np.array_equal(ru[1024:], ra) and np.array_equal(rp[1024:], rpa)
    assert rel(u.cpu(), ru) < tol
    assert rel(p.cpu(), rp) < tolp


@pytest.fixture(scope="module")
def level9(oracle):
    """Icosahedral level 9 (5,242,880 leaf sources in 6,990,500 face slots),
    the C2 initial condition, 2,048 seeded vertices and 2,048 seeded leaf
    centres as passive targets, and the oracle's FP64 velocity there."""
    eps = 0.01
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 9)
    fz = O.ic_eval(O.IC_GAUSSIAN_SPHERE, (4 * math.pi, 4.0, 0.0, 0.05 * math.pi, 0.0, OMEGA), fx)
    iv = sample(vx.shape[0], 2048, 5)
    jf = sample(fx.shape[0], 2048, 6, fm == 0)
    tx = np.concatenate([vx[iv], fx[jf]])
    ru, _ = oracle.ic2d_passive_sums(tx, fx, fz, fa, fm, eps, want_psi=False)
    return tx, fx, fz, fa, fm, eps, ru


@pytest.mark.parametrize("precision,tol", [(core.FP64, 1e-12), (core.FP32C, 1e-6)])
def test_level9_sources(gpu_ctx, level9, precision, tol):
    """The largest source set of the tests: 5.2 M sources (10,240 FP32 tiles,
    hundreds of chunks), so chunk counts, partial offsets and source indices
    run well past the other cases' ranges."""
    ctx = gpu_ctx
    ctx.set_precision(precision)
    tx, fx, fz, fa, fm, eps, ru = level9
    u = zeros(tx.shape[0], 3)
    F.ic2d_passive_sums(ctx, u, None, dev(tx), dev(fx), dev(fz), dev(fa), dev(fm), eps)
    ctx.synchronize()
    assert rel(u.cpu(), ru) < tol


def test_ic2d_dt_conv(gpu_ctx):
    """Second-order time convergence of Incompressible2DRK2 on the GPU."""
    from lpm_gb300.ic2d import Incompressible2D, Incompressible2DRK2

    ctx = gpu_ctx
    ctx.set_precision(core.FP64)
    tf, nsteps = 0.5, (15, 30, 60)
    gauss = (4 * math.pi, 4.0, 0.0, math.pi / 20, 0.0, 0.0)  # GaussianVortexSphere()

    def run(n):
        ic = Incompressible2D(core.MESH_CUBED_SPHERE, 4, eps=0.0, ctx=ctx)
        ic.init_vorticity(core.IC_GAUSSIAN_SPHERE, gauss)
        ic.init_direct_sums()
        solver = Incompressible2DRK2(tf / n, ic, precision=core.FP64)
        for _ in range(n):
            ic.advance_timestep(solver)
        ctx.synchronize()
        return ic.face_x.cpu().numpy(), ic.face_area.cpu().numpy()

    ref, area = run(nsteps[-1])
    errs = [oracle_err(run(n)[0], ref, area) for n in nsteps[:-1]]
    dts = [tf / n for n in nsteps[:-1]]
    for k in range(3):  # l1, l2, linf
        rate = math.log(errs[0][k] / errs[1][k]) / math.log(dts[0] / dts[1])
        assert rate > 1.95, (k, rate)


def oracle_err(appx, exact, wt):
    """ErrNorms of face positions over every face slot (src/lpm_error.hpp:81-91)."""
    return O.err_norms(appx, exact, wt)


@pytest.mark.parametrize("precision,tol", [(core.FP64_CHORD, 1e-11), (core.FP32C, 2e-6)])
def test_c4_ensemble_against_oracle(gpu_ctx, oracle, precision, tol):
    from lpm_gb300.ensemble import BVEEnsemble, random_vortex_params

    ctx = gpu_ctx
    rng = np.random.default_rng(20261203)
    levels = [3, 2]
    params = [random_vortex_params(rng) for _ in levels]
    eps, dt = 0.01, 0.005
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    ens = BVEEnsemble(levels, params, dt, eps=eps, precision=precision, flags=flags, ctx=ctx)
    ens.velocity()
    ctx.synchronize()
    u0 = (ens.vvel.cpu().numpy(), ens.fvel.cpu().numpy())
    for _ in range(2):
        ens.advance_timestep()
    ctx.synchronize()
    with oracle.chord_form():
        for p, (lev, prm) in enumerate(zip(levels, params)):
            vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, lev)
            vz, fz = O.ic_eval(O.IC_MULTI_GAUSSIAN, prm, vx), O.ic_eval(O.IC_MULTI_GAUSSIAN, prm, fx)
            vu, _ = oracle.ic2d_passive_sums(vx, fx, fz, fa, fm, eps, want_psi=False)
            fu, _ = oracle.ic2d_active_sums(fx, fz, fa, fm, eps, self_rule=1)
            vs, fs = ens.problem_slices(p)
            leaf = fm == 0
            assert rel(u0[0][vs], vu) < tol
            assert rel(u0[1][fs][leaf], fu[leaf]) < tol
            ref = oracle.BVEState(vx, vz, vu, fx, fz, fu, fa, fm)
            for _ in range(2):
                ref.step(dt, OMEGA, eps, reproject=True)
            assert rel(ens.vvel[vs].cpu(), ref.vvel) < tol
            assert rel(ens.fvel[fs].cpu().numpy()[leaf], ref.fvel[leaf]) < tol
            assert rel(ens.fx[fs].cpu().numpy()[leaf], ref.fx[leaf]) < tol * 1e-2
            assert rel(ens.fzeta[fs].cpu().numpy()[leaf], ref.fzeta[leaf]) < max(tol, 1e-10)

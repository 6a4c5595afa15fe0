"""Octree far field with the learned correction: tensor-core building block,
gradient check against the CPU oracle, accuracy against the FP64 direct sum
(the reference for its error), the direct-sum fallback, the gain of the trained
network over the expansion alone, and the RK4 stepper on the far field."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mesh(level, ic=("rh",)):
    from lpm_gb300 import core

    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, level, 1.0)
    w = 2 * math.pi / 12.5
    fz = core.eval_ic(core.IC_RH54, (w, -w), fx)
    return vx, fx, fa, fm, fz


def _direct(oracle, x, fx, fz, fa, fm, eps):
    with oracle.chord_form():
        u, _ = oracle.ic2d_passive_sums(x, fx, fz, fa, fm, eps)
    return u


def _ff_velocity(ff, x, fx, fz, fa, fm, eps):
    import torch

    dev = torch.device("cuda", ff.ctx.device)
    X = torch.tensor(x, device=dev)
    U = torch.zeros_like(X)
    ff.velocity(U, X, torch.tensor(fx, device=dev), torch.tensor(fz, device=dev),
                torch.tensor(fa, device=dev), torch.tensor(fm, device=dev), eps)
    torch.cuda.synchronize()
    return U.cpu().numpy()


def _rel_linf(a, b):
    return float(np.max(np.linalg.norm(a - b, axis=1)) / np.max(np.linalg.norm(b, axis=1)))


@pytest.mark.parametrize("amn,bmn,N,K", [(0, 0, 128, 64), (0, 0, 16, 128), (0, 0, 128, 48),
                                         (1, 1, 128, 128), (1, 1, 48, 128), (1, 1, 16, 128),
                                         (0, 1, 128, 16)])
def test_tcgen05_gemm(gpu_ctx, amn, bmn, N, K):
    """Every operand arrangement the network kernels use, against numpy."""
    import torch
    from mlp_oracle import bf16

    from lpm_gb300.farfield import tc_selftest

    rng = np.random.default_rng(N * 1000 + K + 7 * amn + 13 * bmn)
    A = rng.uniform(-1, 1, (K, 128) if amn else (128, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N) if bmn else (N, K)).astype(np.float32)
    dev = torch.device("cuda", gpu_ctx.device)
    D = tc_selftest(gpu_ctx, torch.tensor(A, device=dev), torch.tensor(B, device=dev), N, K,
                    bool(amn), bool(bmn)).cpu().numpy()
    Ab, Bb = bf16(A), bf16(B)
    ref = (Ab.T if amn else Ab) @ (Bb if bmn else Bb.T)
    assert np.max(np.abs(D - ref)) <= 1e-5 * np.max(np.abs(ref))


def _rand_net(seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(40960, np.float32)
    off = 0
    for rows, cols, fan, live, bias in ((128, 48, 40, 127, 40), (128, 128, 127, 127, 127),
                                        (128, 128, 127, 127, 127), (16, 128, 127, 3, 127)):
        m = rng.uniform(-1, 1, (rows, cols)) / math.sqrt(fan)
        m[live:, :] = 0
        m[:live, bias] = rng.uniform(-0.1, 0.1, live)
        w[off:off + rows * cols] = m.ravel()
        off += rows * cols
    return w


def test_gradient_matches_oracle(gpu_ctx):
    """Gradients of the tcgen05 training kernel vs the FP64 oracle with the
    same BF16 rounding points (relative L2 per matrix)."""
    import mlp_oracle as mo

    from lpm_gb300.farfield import FarField

    ff = FarField(ctx=gpu_ctx)
    w = _rand_net(3)
    ff.set_weights(w, np.concatenate([np.zeros(48), np.ones(48), [1.0]]).astype(np.float32))
    rng = np.random.default_rng(5)
    n = 256
    x = rng.normal(0, 1, (n, 48)).astype(np.float32)
    x[:, 40] = 1.0
    x[:, 41:] = 0.0
    x = mo.bf16(x).astype(np.float32)
    y = rng.normal(0, 0.5, (n, 3)).astype(np.float32)
    g = ff.grad(x, y).astype(np.float64)
    r = mo.grad(w, x, y)
    offs = [0, 128 * 48, 128 * 48 + 128 * 128, 128 * 48 + 2 * 128 * 128, 40960]
    for a, b in zip(offs[:-1], offs[1:]):
        err = np.linalg.norm(g[a:b] - r[a:b]) / np.linalg.norm(r[a:b])
        assert err < 2e-2, (a, err)


def test_treecode_accuracy_and_convergence(gpu_ctx, oracle):
    """Order-4 expansion + exact near field vs the FP64 direct sum; the error
    falls with the opening angle."""
    from lpm_gb300.farfield import FarField

    vx, fx, fa, fm, fz = _mesh(5)
    eps = 0.01
    x = np.concatenate([vx, fx[fm == 0]])
    ref = _direct(oracle, x, fx, fz, fa, fm, eps)
    errs = {}
    for theta in (0.5, 0.3):
        ff = FarField(theta=theta, ctx=gpu_ctx)
        u = _ff_velocity(ff, x, fx, fz, fa, fm, eps)
        errs[theta] = _rel_linf(u, ref)
        st = ff.stats()
        assert st["fallback_blocks"] == 0 and st["far_pairs"] > 0
    assert errs[0.5] < 1e-3, errs
    assert errs[0.3] < errs[0.5] / 3, errs


def test_direct_sum_fallback(gpu_ctx, oracle):
    """A tiny opening angle overflows the near lists (level 7: 15,694 leaves
    against 4,096 list entries): the blocks fall back to the exact direct sum
    (FP32 compensated)."""
    from lpm_gb300.farfield import FarField

    vx, fx, fa, fm, fz = _mesh(7)
    x = np.ascontiguousarray(vx[::64])
    eps = 0.01
    ff = FarField(theta=0.02, rho_min=0.01, ctx=gpu_ctx)
    u = _ff_velocity(ff, x, fx, fz, fa, fm, eps)
    assert ff.stats()["fallback_blocks"] > 0
    ref = _direct(oracle, x, fx, fz, fa, fm, eps)
    assert _rel_linf(u, ref) < 2e-6


def test_learned_correction_gains(gpu_ctx, oracle):
    """Train on seeded random vortex fields; on a held-out Rossby-Haurwitz
    field the network reduces the far-field error of the expansion."""
    from lpm_gb300.farfield import FarField

    ff = FarField(theta=0.5, ctx=gpu_ctx)
    loss = ff.train(nsamples=1 << 22, epochs=6, batch=16384, lr=2e-3, seed=11, level_min=5,
                    level_max=8, eps=0.01)
    assert all(np.isfinite(loss)) and loss[-1] < loss[0]
    vx, fx, fa, fm, fz = _mesh(7)
    eps = 0.01
    x = vx[::8]
    ref = _direct(oracle, x, fx, fz, fa, fm, eps)
    ff.set_network(False)
    e0 = _rel_linf(_ff_velocity(ff, x, fx, fz, fa, fm, eps), ref)
    ff.set_network(True)
    e1 = _rel_linf(_ff_velocity(ff, x, fx, fz, fa, fm, eps), ref)
    st = ff.stats()
    assert st["learned_pairs"] > 0 and 0 < st["network_rows"] <= 128 * st["learned_pairs"]
    assert e1 < 0.8 * e0, (e0, e1)
    # weights round-trip through the host
    w, nrm = ff.get_weights()
    ff2 = FarField(theta=0.5, ctx=gpu_ctx)
    ff2.set_weights(w, nrm)
    ff2.set_network(True)
    e2 = _rel_linf(_ff_velocity(ff2, x, fx, fz, fa, fm, eps), ref)
    assert e2 == pytest.approx(e1, rel=1e-9)


def test_rk4_step_on_farfield(gpu_ctx):
    """One BVERK4 step evaluated by the far field stays close to the same step
    with the FP64 chord-form direct sum."""
    import ctypes as C

    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F
    from lpm_gb300.farfield import FarField

    eps, dt = 0.01, 0.005
    vx, fx, fa, fm, fz = _mesh(5)
    vz = core.eval_ic(core.IC_RH54, (2 * math.pi / 12.5, -2 * math.pi / 12.5), vx)
    dev = torch.device("cuda", gpu_ctx.device)
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    out = []
    keep = []
    for use_ff in (False, True):
        t = {k: torch.tensor(v, device=dev) for k, v in
             dict(vx=vx, fx=fx, fa=fa, fm=fm, fz=fz, vz=vz).items()}
        vu = torch.zeros_like(t["vx"])
        fu = torch.zeros_like(t["fx"])
        F.ic2d_passive_sums(gpu_ctx, vu, None, t["vx"], t["fx"], t["fz"], t["fa"], t["fm"], eps)
        F.ic2d_passive_sums(gpu_ctx, fu, None, t["fx"], t["fx"], t["fz"], t["fa"], t["fm"], eps)
        h = C.c_void_p()
        core.check(core.lib().lpm_bve_rk4_create(gpu_ctx.handle, C.byref(h), vx.shape[0],
                                                 fx.shape[0], dt, 2 * math.pi, eps,
                                                 core.FP64_CHORD, flags))
        if use_ff:
            ff = FarField(theta=0.5, ctx=gpu_ctx)
            keep.append(ff)
            core.check(core.lib().lpm_bve_rk4_set_farfield(h, ff.handle, 0))
        core.check(core.lib().lpm_bve_rk4_advance_timestep(
            h, core.view(t["vx"]), core.ptr(t["vz"]), core.view(vu), core.view(t["fx"]),
            core.ptr(t["fz"]), core.view(fu), core.ptr(t["fa"]), core.ptr(t["fm"])))
        torch.cuda.synchronize()
        leaf = fm == 0
        out.append((t["fx"].cpu().numpy()[leaf], fu.cpu().numpy()[leaf], t["fz"].cpu().numpy()[leaf]))
        core.lib().lpm_bve_rk4_destroy(h)
    (x0, u0, z0), (x1, u1, z1) = out
    assert np.max(np.abs(x1 - x0)) < 1e-5
    assert _rel_linf(u1, u0) < 2e-3
    assert np.max(np.abs(z1 - z0)) < 1e-4 * np.max(np.abs(z0))


def test_argument_errors(gpu_ctx):
    from lpm_gb300.core import LpmError
    from lpm_gb300.farfield import FarField

    with pytest.raises(LpmError):
        FarField(theta=1.5, ctx=gpu_ctx)
    with pytest.raises(LpmError):
        FarField(leaf_max=65, ctx=gpu_ctx)
    ff = FarField(ctx=gpu_ctx)
    with pytest.raises(LpmError):
        ff.set_network(True)  # nothing trained or loaded
    with pytest.raises(LpmError):
        ff.stats()  # no evaluation yet


def test_farfield_deterministic_and_strided_views(gpu_ctx):
    """Two evaluations with the network give bitwise equal results; targets
    and outputs in a component-major (Kokkos LayoutLeft) layout give the same
    velocities as row-major ones."""
    import torch

    from lpm_gb300.farfield import FarField

    vx, fx, fa, fm, fz = _mesh(5)
    eps = 0.01
    ff = FarField(ctx=gpu_ctx)
    ff.set_weights(_rand_net(7) * 0.1,
                   np.concatenate([np.zeros(48), np.ones(48), [1e-3]]).astype(np.float32))
    ff.set_network(True)
    u1 = _ff_velocity(ff, vx, fx, fz, fa, fm, eps)
    u2 = _ff_velocity(ff, vx, fx, fz, fa, fm, eps)
    assert np.array_equal(u1, u2)
    assert ff.stats()["network_rows"] > 0
    d = torch.device("cuda", gpu_ctx.device)
    xl = torch.tensor(np.ascontiguousarray(vx.T), device=d).t()   # strides (1, n)
    ul = torch.zeros(3, vx.shape[0], dtype=torch.float64, device=d).t()
    fxl = torch.tensor(np.ascontiguousarray(fx.T), device=d).t()
    ff.velocity(ul, xl, fxl, torch.tensor(fz, device=d), torch.tensor(fa, device=d),
                torch.tensor(fm, device=d), eps)
    torch.cuda.synchronize()
    assert np.array_equal(ul.cpu().numpy(), u1)


def test_rk4_farfield_rebuilds_tree(gpu_ctx):
    """A stepper that rebuilds its tree every step stays within the far
    field's error of one that keeps the first tree."""
    import ctypes as C

    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F
    from lpm_gb300.farfield import FarField

    eps, dt = 0.01, 0.005
    vx, fx, fa, fm, fz = _mesh(4)
    vz = core.eval_ic(core.IC_RH54, (2 * math.pi / 12.5, -2 * math.pi / 12.5), vx)
    d = torch.device("cuda", gpu_ctx.device)
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    out, keep = [], []
    for every in (0, 1):
        t = {k: torch.tensor(v, device=d) for k, v in
             dict(vx=vx, fx=fx, fa=fa, fm=fm, fz=fz, vz=vz).items()}
        vu, fu = torch.zeros_like(t["vx"]), torch.zeros_like(t["fx"])
        F.ic2d_passive_sums(gpu_ctx, vu, None, t["vx"], t["fx"], t["fz"], t["fa"], t["fm"], eps)
        F.ic2d_passive_sums(gpu_ctx, fu, None, t["fx"], t["fx"], t["fz"], t["fa"], t["fm"], eps)
        h = C.c_void_p()
        core.check(core.lib().lpm_bve_rk4_create(gpu_ctx.handle, C.byref(h), vx.shape[0],
                                                 fx.shape[0], dt, 2 * math.pi, eps,
                                                 core.FP64_CHORD, flags))
        ff = FarField(ctx=gpu_ctx)
        keep.append(ff)
        core.check(core.lib().lpm_bve_rk4_set_farfield(h, ff.handle, every))
        for _ in range(3):
            core.check(core.lib().lpm_bve_rk4_advance_timestep(
                h, core.view(t["vx"]), core.ptr(t["vz"]), core.view(vu), core.view(t["fx"]),
                core.ptr(t["fz"]), core.view(fu), core.ptr(t["fa"]), core.ptr(t["fm"])))
        torch.cuda.synchronize()
        out.append(fu.cpu().numpy()[fm == 0])
        core.lib().lpm_bve_rk4_destroy(h)
    assert _rel_linf(out[1], out[0]) < 2e-3

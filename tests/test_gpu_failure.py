"""Failure handling and restart on the GPU, without faulting it.

- A bounded wait that runs out: lpm_wait_selftest arms a tile mbarrier for a
  copy that is never issued; after its poll limit the CTA flags the error and
  returns.  lpm_context_synchronize reports LPM_ERR_TIMEOUT once, and the same
  context then computes correct sums.
- The entry points leave the calling thread's current device as they found
  it (one GPU here: the context's device is the current one).
- Checkpoint / restart: two RK4 steps, a snapshot of the particle state to a
  file, a new BVESphere and BVERK4 from it and two more steps equal four
  uninterrupted steps bit for bit.
"""
import ctypes as C
import math

import numpy as np
import pytest
import torch

import lpm_oracle as O
from lpm_gb300 import core
from lpm_gb300 import functors as F
from lpm_gb300.bve import BVERK4, BVESphere, rossby_haurwitz_params

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_recovers(gpu_ctx, oracle):
    ctx = gpu_ctx
    L = core.lib()
    assert L.lpm_wait_selftest(ctx.handle, 0) == core.LPM_ERR_ARG
    assert L.lpm_wait_selftest(ctx.handle, 512) == core.LPM_OK
    rc = L.lpm_context_synchronize(ctx.handle)
    assert rc == core.LPM_ERR_TIMEOUT
    assert b"bounded device-side wait" in L.lpm_last_error()
    assert L.lpm_context_synchronize(ctx.handle) == core.LPM_OK  # the flag was cleared
    # the same context still computes correct sums
    ctx.set_precision(core.FP64)
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 3)
    fz = O.ic_eval(O.IC_RH54, (0.5, -0.5), fx)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
    F.bve_vertex_velocity(ctx, u, d(vx), d(fx), d(fz), d(fa), d(fm))
    assert L.lpm_context_synchronize(ctx.handle) == core.LPM_OK
    _, ref = oracle.bve_vertex_solve(vx, fx, fz, fa, fm, want_psi=False)
    assert np.abs(u.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


def test_current_device_unchanged(gpu_ctx):
    from lpm_gb300.core import check, crd3, lib, ptr

    before = torch.cuda.current_device()
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2)
    T = {k: torch.tensor(v, device="cuda") for k, v in dict(vx=vx, fx=fx, fa=fa, fm=fm).items()}
    z = torch.ones(fx.shape[0], dtype=torch.float64, device="cuda")
    u = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
    check(lib().lpm_bve_direct_sum(crd3(T["vx"]), crd3(T["fx"]), ptr(z), ptr(T["fa"]),
                                   ptr(T["fm"]), fx.shape[0], 0, 0.0, 1, core.FP64, ptr(u), 3, 1,
                                   None, None))
    torch.cuda.synchronize()
    check(lib().lpm_one_call_release())
    assert torch.cuda.current_device() == before


@pytest.mark.parametrize("precision", [core.FP64, core.FP32C])
def test_checkpoint_restart_is_bitwise(gpu_ctx, tmp_path, precision):
    ctx = gpu_ctx
    ctx.set_precision(precision)

    def fresh():
        s = BVESphere(3, ctx=ctx)
        s.init_vorticity(core.IC_RH54, rossby_haurwitz_params())
        s.init_velocity()
        return s

    a = fresh()
    sa = BVERK4(0.01, a, precision=precision)
    for _ in range(4):
        sa.advance_timestep(a)
    b = fresh()
    sb = BVERK4(0.01, b, precision=precision)
    for _ in range(2):
        sb.advance_timestep(b)
    ctx.synchronize()
    b.save(tmp_path / "state.npz")
    sb.close()
    del b
    c = BVESphere.from_snapshot(tmp_path / "state.npz", ctx=ctx)
    sc = BVERK4(0.01, c, precision=precision)
    for _ in range(2):
        sc.advance_timestep(c)
    ctx.synchronize()
    for k in BVESphere._STATE:
        assert torch.equal(getattr(a, k), getattr(c, k)), k
    assert math.isclose(a.t, c.t, rel_tol=0, abs_tol=1e-15) and a.Omega == c.Omega

"""The allocation-free entry point lpm_bve_vertex_velocity_static.

It serves callers that cannot call cudaMalloc (device memory owned by another
allocator or a fixed budget, or host loops that must not stall on the device
synchronisation cudaMalloc/cudaFree can cause).  Here it is checked against
the regular lpm_bve_vertex_velocity (which allocates its scratch) in the same
FP32-compensated arithmetic, on two calls in a row with different inputs, so
the shared scratch array cannot carry state from one call into the next.

This file is named to be collected last.
"""
import math

import numpy as np
import pytest
import torch

from lpm_gb300 import core
from lpm_gb300 import functors as F

pytestmark = pytest.mark.gpu

TOL32 = 2e-6


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


def case(level, seed):
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, level, 1.0)
    w = 2 * math.pi / 12.5
    zf = core.eval_ic(core.IC_RH54, (w, -w), fx)
    zf = zf + 0.3 * np.random.default_rng(seed).standard_normal(zf.shape)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return dev(vx), dev(fx), dev(zf), dev(fa), dev(fm)


def static_call(u, vx, fx, zf, fa, fm, stream):
    return core.lib().lpm_bve_vertex_velocity_static(
        core.view(u), core.view(vx), vx.shape[0], core.view(fx), core.ptr(zf), core.ptr(fa),
        core.ptr(fm), fx.shape[0], stream)


def test_static_scratch_matches_regular_entry_point():
    from lpm_gb300 import build as B

    B.build()
    ctx = core.Context(0, precision=core.FP32C)
    stream = torch.cuda.current_stream().cuda_stream
    ctx.set_stream(torch.cuda.current_stream())
    free_after = []
    # calls in a row with different sizes; at level 7 the chunk partials of
    # an unconstrained plan (about 40 chunks x 3 x 164,864 targets x 8 B, over
    # 150 MB) do not fit the 64 MiB array, so the plan's chunk count is the
    # one the array's remaining bytes allow
    for level, seed in ((7, 1), (4, 2), (3, 3)):
        vx, fx, zf, fa, fm = case(level, seed)
        u_static = torch.full((vx.shape[0], 3), float("nan"), dtype=torch.float64,
                              device="cuda")
        core.check(static_call(u_static, vx, fx, zf, fa, fm, stream))
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
        u_ref = torch.zeros_like(u_static)
        F.bve_vertex_velocity(ctx, u_ref, vx, fx, zf, fa, fm)
        ctx.synchronize()
        assert torch.isfinite(u_static).all()
        assert rel(u_static.cpu(), u_ref.cpu()) < TOL32
    # the second call allocated nothing on the device (torch's cache is idle
    # between the two reads, and the library's own arena grew only in the
    # regular call, before the second static call)
    vx, fx, zf, fa, fm = case(3, 2)
    u2 = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
    # free device memory is a device-wide figure: another process may
    # allocate in between, so one unequal reading is measured again
    for attempt in range(2):
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info()[0]
        core.check(static_call(u2, vx, fx, zf, fa, fm, stream))
        torch.cuda.synchronize()
        if torch.cuda.mem_get_info()[0] == before:
            break
    else:
        pytest.fail("free device memory changed across two static calls")


def test_static_scratch_rejects_oversized_problems():
    vx, fx, zf, fa, fm = case(1, 3)
    u = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
    # counts far beyond the 64 MiB scratch: rejected before any memory is read
    rc = core.lib().lpm_bve_vertex_velocity_static(
        core.view(u), core.view(vx), 4_000_000, core.view(fx), core.ptr(zf), core.ptr(fa),
        core.ptr(fm), 4_000_000, None)
    assert rc == core.LPM_ERR_ARG
    assert b"static scratch holds" in core.lib().lpm_last_error()

"""Ensemble stepper: each problem advanced inside the ensemble (one N-body
launch per evaluation for all problems, persistent or one CTA per work item)
matches the same problem advanced alone by BVERK4 in the same arithmetic."""
import math

import numpy as np
import pytest
import torch

from lpm_gb300 import core
from lpm_gb300 import functors as F
from lpm_gb300.bve import BVERK4, BVESphere
from lpm_gb300.ensemble import BVEEnsemble, random_vortex_params

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("precision,tol", [(core.FP64_CHORD, 1e-11), (core.FP32C, 2e-6)])
def test_ensemble_matches_single_problems(gpu_ctx, precision, tol):
    ctx = gpu_ctx
    rng = np.random.default_rng(20261203)
    levels = [2, 0, 3, 1, 2, 3]
    params = [random_vortex_params(rng) for _ in levels]
    eps, dt = 0.01, 0.005
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    ens = BVEEnsemble(levels, params, dt, eps=eps, precision=precision, flags=flags, ctx=ctx)
    ens.velocity()
    for _ in range(2):
        ens.advance_timestep()
    ctx.synchronize()
    info = ens.info()
    assert info["chunk_len"] > 0 and info["items"] > 0
    for p, (lev, prm) in enumerate(zip(levels, params)):
        sph = BVESphere(lev, ctx=ctx)
        sph.init_vorticity(core.IC_MULTI_GAUSSIAN, prm)
        ctx.set_precision(precision)
        F.ic2d_passive_sums(ctx, sph.velocity_verts, None, sph.vert_x, sph.face_x,
                            sph.rel_vort_faces, sph.face_area, sph.face_mask, eps)
        F.ic2d_active_sums(ctx, sph.velocity_faces, None, sph.face_x, sph.rel_vort_faces,
                           sph.face_area, sph.face_mask, eps, self_rule=1)
        st = BVERK4(dt, sph, precision=precision, eps=eps, flags=flags)
        for _ in range(2):
            st.advance_timestep(sph)
        ctx.synchronize()
        vs, fs = ens.problem_slices(p)
        leaf = sph.host_face_mask == 0
        assert rel(ens.vvel[vs].cpu(), sph.velocity_verts.cpu()) < tol
        assert rel(ens.fvel[fs].cpu().numpy()[leaf], sph.velocity_faces.cpu().numpy()[leaf]) < tol
        assert rel(ens.fx[fs].cpu().numpy()[leaf], sph.face_x.cpu().numpy()[leaf]) < tol * 1e-2
        assert rel(ens.fzeta[fs].cpu().numpy()[leaf],
                   sph.rel_vort_faces.cpu().numpy()[leaf]) < max(tol, 1e-10)


def test_ensemble_graph_replay_is_deterministic(gpu_ctx):
    ctx = gpu_ctx
    rng = np.random.default_rng(7)
    levels = [3, 2, 4]
    params = [random_vortex_params(rng) for _ in levels]
    outs = []
    for flags in (core.STEP_SKIP_MASKED_TARGETS, core.STEP_SKIP_MASKED_TARGETS | core.STEP_NO_GRAPH):
        ens = BVEEnsemble(levels, params, 0.005, eps=0.01, flags=flags, ctx=ctx)
        ens.set_chunk_len(2048)
        ens.velocity()
        for _ in range(3):
            ens.advance_timestep()
        ctx.synchronize()
        outs.append((ens.fx.clone(), ens.fvel.clone()))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])


def test_ensemble_kernel_forms_agree(gpu_ctx):
    """Every kernel shape, persistent or one CTA per work item, gives the
    same velocities bit for bit at a fixed chunk length."""
    ctx = gpu_ctx
    rng = np.random.default_rng(3)
    levels = [3, 1, 4, 2]
    params = [random_vortex_params(rng) for _ in levels]
    outs = []
    for shape in range(6):
        for persistent in (True, False):
            ens = BVEEnsemble(levels, params, 0.005, eps=0.01, flags=core.STEP_SKIP_MASKED_TARGETS,
                              ctx=ctx)
            ens.set_kernel(shape, persistent)
            ens.set_chunk_len(2048)
            ens.velocity()
            ctx.synchronize()
            assert ens.shape()[2] == persistent
            outs.append((ens.vvel.clone(), ens.fvel.clone()))
            ens.close()
    for o in outs[1:]:
        assert torch.equal(outs[0][0], o[0]) and torch.equal(outs[0][1], o[1])


def test_ensemble_c4_scale(gpu_ctx):
    """64 problems drawn like the C4 workload (levels 3-6, 1-4 Gaussian
    vortices each), the plan autotuned over chunk length, the six kernel
    shapes and both launch forms (thousands of work items): one evaluation
    agrees with each sampled problem evaluated alone, FP32C against FP32C
    (different chunkings: 2e-6)."""
    ctx = gpu_ctx
    rng = np.random.default_rng(20261204)
    levels = [int(v) for v in rng.integers(3, 7, size=64)]
    params = [random_vortex_params(rng) for _ in levels]
    eps = 0.01
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    ens = BVEEnsemble(levels, params, 0.005, eps=eps, precision=core.FP32C, flags=flags, ctx=ctx)
    ens.velocity()
    ctx.synchronize()
    info = ens.info()
    assert info["items"] > 1000 and info["chunk_len"] % 512 == 0
    picks = [int(np.argmax(levels)), int(np.argmin(levels)), 31]
    for p in picks:
        sph = BVESphere(levels[p], ctx=ctx)
        sph.init_vorticity(core.IC_MULTI_GAUSSIAN, params[p])
        ctx.set_precision(core.FP32C)
        F.ic2d_passive_sums(ctx, sph.velocity_verts, None, sph.vert_x, sph.face_x,
                            sph.rel_vort_faces, sph.face_area, sph.face_mask, eps)
        F.ic2d_active_sums(ctx, sph.velocity_faces, None, sph.face_x, sph.rel_vort_faces,
                           sph.face_area, sph.face_mask, eps, self_rule=1)
        ctx.synchronize()
        vs, fs = ens.problem_slices(p)
        leaf = sph.host_face_mask == 0
        assert rel(ens.vvel[vs].cpu(), sph.velocity_verts.cpu()) < 2e-6, p
        assert rel(ens.fvel[fs].cpu().numpy()[leaf], sph.velocity_faces.cpu().numpy()[leaf]) < 2e-6, p
    ens.close()

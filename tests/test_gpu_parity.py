"""CUDA path vs the FP64 CPU oracle on the same inputs (run with -m gpu).

Tolerances (relative to the largest reference magnitude, the ErrNorms linf
normalisation of src/lpm_error.hpp:81-91):
  FP64_EXACT  1e-12 on every target (each pair term is bit-identical; only
              the grouping of the sum differs), non-finite entries matched
  FP64        1e-12 on vertices and leaf faces (cross product out of the sum,
              Newton-Raphson quotients); at a divided parent slot whose centre
              coincides with its central child's, the reference's value is
              non-finite and the hoisted form's is not defined either
  FP32C path  2e-6 velocity, 2e-6 stream function on leaf targets
"""
import math

import numpy as np
import pytest
import torch

from lpm_gb300 import core
from lpm_gb300 import functors as F

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL64C = 1e-11  # FP64 chord form vs the chord-form oracle (different operation order)
TOL32 = 2e-6
OMEGA = 2 * math.pi


def rel(a, b):
    """max|a-b| / max|b| over finite entries; the non-finite entries must match.

    The reference's FP64 arithmetic divides by zero at a divided parent slot
    whose centre coincides with its central child's centre (1 - x.y == 0), so
    both the oracle and the FP64 path give inf/nan there."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), "non-finite entries differ"
    a, b = a[fb], b[fb]
    if b.size == 0:
        return 0.0
    den = np.abs(b).max()
    return np.abs(a - b).max() / (den if den > 0 else 1.0)


def same(a, b):
    """Bitwise-equal finite values and the same non-finite pattern."""
    fa, fb = torch.isfinite(a), torch.isfinite(b)
    return torch.equal(fa, fb) and torch.equal(a[fa], b[fb])


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def sphere_case(level, seed=core.MESH_ICOS_TRI, kind=core.IC_RH54, params=None, noise=0.0):
    vx, fx, fa, fm = core.build_mesh(seed, level, 1.0)
    if params is None:
        w = OMEGA / 12.5
        params = (w, -w)
    zf = core.eval_ic(kind, params, fx)
    if noise:
        zf = zf + noise * np.random.default_rng(7).standard_normal(zf.shape)
    return vx, fx, fa, fm, zf


def tolerance(precision):
    return {core.FP64: TOL64, core.FP64_EXACT: TOL64, core.FP64_CHORD: TOL64C,
            core.FP32C: TOL32}[precision]


REF_FORM = (core.FP64, core.FP64_EXACT)


@pytest.mark.parametrize("level", [0, 2, 3])
@pytest.mark.parametrize("precision", [core.FP64, core.FP64_EXACT, core.FP64_CHORD, core.FP32C])
def test_bve_functors(gpu_ctx, oracle, level, precision):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    vx, fx, fa, fm, zf = sphere_case(level, noise=0.5)
    oracle.set_sphere_form(precision not in REF_FORM)
    try:
        psi_v, u_v = oracle.bve_vertex_solve(vx, fx, zf, fa, fm)
        psi_f, u_f = oracle.bve_face_solve(fx, zf, fa, fm)
    finally:
        oracle.set_sphere_form(False)
    dvx, dfx, dz, da, dm = dev(vx), dev(fx), dev(zf), dev(fa), dev(fm)
    gu = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
    gp = torch.zeros(vx.shape[0], dtype=torch.float64, device="cuda")
    F.bve_vertex_solve(ctx, gp, gu, dvx, dfx, dz, da, dm)
    gfu = torch.zeros(fx.shape[0], 3, dtype=torch.float64, device="cuda")
    gfp = torch.zeros(fx.shape[0], dtype=torch.float64, device="cuda")
    F.bve_face_solve(ctx, gfp, gfu, dfx, dz, da, dm)
    ctx.synchronize()
    leaf = fm == 0
    if precision == core.FP64_EXACT:
        assert rel(gu.cpu(), u_v) < TOL64
        assert rel(gp.cpu(), psi_v) < TOL64
        assert rel(gfu.cpu(), u_f) < TOL64
        assert rel(gfp.cpu(), psi_f) < TOL64
    else:
        tol = tolerance(precision)
        assert rel(gu.cpu(), u_v) < tol
        assert rel(gp.cpu(), psi_v) < tol
        assert rel(gfu.cpu().numpy()[leaf], u_f[leaf]) < tol
        assert rel(gfp.cpu().numpy()[leaf], psi_f[leaf]) < tol
    # velocity-only and stream-function-only launches give the same values
    gu2 = torch.zeros_like(gu)
    F.bve_vertex_velocity(ctx, gu2, dvx, dfx, dz, da, dm)
    gp2 = torch.zeros_like(gp)
    F.bve_vertex_stream_fn(ctx, gp2, dvx, dfx, dz, da, dm)
    gfu2 = torch.zeros_like(gfu)
    F.bve_face_velocity(ctx, gfu2, dfx, dz, da, dm)
    gfp2 = torch.zeros_like(gfp)
    F.bve_face_stream_fn(ctx, gfp2, dfx, dz, da, dm)
    ctx.synchronize()
    assert same(gu2, gu) and same(gfu2, gfu)
    tolp = 0 if precision in REF_FORM else 1e-12
    assert rel(gp2.cpu(), gp.cpu()) <= tolp and rel(gfp2.cpu(), gfp.cpu()) <= tolp


def test_bve_soa_layout(gpu_ctx, oracle):
    """LayoutLeft (SoA, stride = nmax) views give the same answer as AoS."""
    ctx = gpu_ctx
    ctx.set_precision(core.FP64)
    vx, fx, fa, fm, zf = sphere_case(3)
    nmax_v, nmax_f = vx.shape[0] + 5, fx.shape[0] + 3
    soa_v = torch.zeros(3, nmax_v, dtype=torch.float64, device="cuda")
    soa_v[:, : vx.shape[0]] = dev(vx).T
    soa_f = torch.zeros(3, nmax_f, dtype=torch.float64, device="cuda")
    soa_f[:, : fx.shape[0]] = dev(fx).T
    vview = soa_v[:, : vx.shape[0]].T  # stride (1, nmax)
    fview = soa_f[:, : fx.shape[0]].T
    assert vview.stride() == (1, nmax_v)
    u_soa = torch.zeros(3, nmax_v, dtype=torch.float64, device="cuda")
    F.bve_vertex_velocity(ctx, u_soa[:, : vx.shape[0]].T, vview, fview, dev(zf), dev(fa), dev(fm))
    _, u_ref = oracle.bve_vertex_solve(vx, fx, zf, fa, fm, want_psi=False)
    ctx.synchronize()
    assert rel(u_soa[:, : vx.shape[0]].T.cpu(), u_ref) < TOL64


@pytest.mark.parametrize("eps", [0.0, 0.05])
@pytest.mark.parametrize("precision", [core.FP64, core.FP64_EXACT, core.FP64_CHORD, core.FP32C])
@pytest.mark.parametrize("geom", ["sphere", "plane"])
def test_ic2d_functors(gpu_ctx, oracle, eps, precision, geom):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    if geom == "sphere":
        vx, fx, fa, fm, zf = sphere_case(3, seed=core.MESH_CUBED_SPHERE,
                                         kind=core.IC_GAUSSIAN_SPHERE,
                                         params=(4 * math.pi, 4.0, 0.0, math.pi / 20, 0.0, 0.0))
    else:
        vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, 4, 4.0)
        zf = core.eval_ic(core.IC_DIPOLE_PAIR, (2.0, 1.0, -2.0, 0.0, -2.0, 1.0, 2.0, 0.0), fx)
    nd = vx.shape[1]
    oracle.set_sphere_form(precision not in REF_FORM)
    try:
        u_p, psi_p = oracle.ic2d_passive_sums(vx, fx, zf, fa, fm, eps)
        u_a, psi_a = oracle.ic2d_active_sums(fx, zf, fa, fm, eps)
    finally:
        oracle.set_sphere_form(False)
    gu = torch.zeros(vx.shape[0], nd, dtype=torch.float64, device="cuda")
    gp = torch.zeros(vx.shape[0], dtype=torch.float64, device="cuda")
    fu = torch.zeros(fx.shape[0], nd, dtype=torch.float64, device="cuda")
    fp = torch.zeros(fx.shape[0], dtype=torch.float64, device="cuda")
    dfx, dz, da, dm = dev(fx), dev(zf), dev(fa), dev(fm)
    F.ic2d_passive_sums(ctx, gu, gp, dev(vx), dfx, dz, da, dm, eps)
    F.ic2d_active_sums(ctx, fu, fp, dfx, dz, da, dm, eps)
    ctx.synchronize()
    leaf = fm == 0
    tol = tolerance(precision)
    assert rel(gu.cpu(), u_p) < tol
    assert rel(gp.cpu(), psi_p) < tol
    sel = slice(None) if precision == core.FP64_EXACT else leaf
    assert rel(fu.cpu().numpy()[sel], u_a[sel]) < tol
    assert rel(fp.cpu().numpy()[sel], psi_a[sel]) < tol


@pytest.mark.parametrize("precision", [core.FP64, core.FP32C])
def test_edge_cases(gpu_ctx, oracle, precision):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    vx, fx, fa, fm, zf = sphere_case(1)
    dfx, dz, da = dev(fx), dev(zf), dev(fa)
    # every face masked: no sources, all sums zero
    allm = torch.ones(fx.shape[0], dtype=torch.uint8, device="cuda")
    u = torch.full((vx.shape[0], 3), 7.0, dtype=torch.float64, device="cuda")
    F.bve_vertex_velocity(ctx, u, dev(vx), dfx, dz, da, allm)
    ctx.synchronize()
    assert torch.count_nonzero(u) == 0
    # a single target, a single unmasked source
    one = np.ones(fx.shape[0], np.uint8)
    one[fx.shape[0] - 1] = 0
    u1 = torch.zeros(1, 3, dtype=torch.float64, device="cuda")
    F.bve_vertex_velocity(ctx, u1, dev(vx[:1]), dfx, dz, da, dev(one))
    _, ur = oracle.bve_vertex_solve(vx[:1], fx, zf, fa, one, want_psi=False)
    ctx.synchronize()
    assert rel(u1.cpu(), ur) < (TOL64 if precision == core.FP64 else TOL32)
    # zero targets: no launch, no error
    u0 = torch.zeros(0, 3, dtype=torch.float64, device="cuda")
    F.bve_vertex_velocity(ctx, u0, dev(vx[:0]), dfx, dz, da, dev(fm))
    ctx.synchronize()


def test_determinism(gpu_ctx):
    ctx = gpu_ctx
    for precision in (core.FP64, core.FP32C):
        ctx.set_precision(precision)
        vx, fx, fa, fm, zf = sphere_case(4)
        outs = []
        for _ in range(2):
            u = torch.zeros(fx.shape[0], 3, dtype=torch.float64, device="cuda")
            F.bve_face_velocity(ctx, u, dev(fx), dev(zf), dev(fa), dev(fm))
            outs.append(u)
        ctx.synchronize()
        assert same(outs[0], outs[1])


@pytest.mark.parametrize("geom,eps", [("sphere", 0.01), ("plane", 0.02), ("plane", 0.0)])
def test_fp32_kernel_shapes_agree(gpu_ctx, oracle, geom, eps):
    """Every FP32 kernel shape gives the same bits (each target is summed by
    one thread in source order, with the same operations whatever the
    shape), and each is within the FP32C tolerance of the oracle."""
    ctx = gpu_ctx
    ctx.set_precision(core.FP32C)
    if geom == "sphere":
        vx, fx, fa, fm, zf = sphere_case(4)
    else:
        vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, 5, 4.0)
        zf = core.eval_ic(core.IC_DIPOLE_PAIR, (2.0, 1.0, -2.0, 0.0, -2.0, 1.0, 2.0, 0.0), fx)
    nd = vx.shape[1]
    dvx, dfx, dz, da, dm = dev(vx), dev(fx), dev(zf), dev(fa), dev(fm)
    outs = []
    try:
        for shape in range(6):
            ctx.set_kernel_shape(shape)
            u = torch.zeros(vx.shape[0], nd, dtype=torch.float64, device="cuda")
            p = torch.zeros(vx.shape[0], dtype=torch.float64, device="cuda")
            F.ic2d_passive_sums(ctx, u, p, dvx, dfx, dz, da, dm, eps)
            outs.append((u, p))
        ctx.synchronize()
    finally:
        ctx.set_kernel_shape(-1)
    for u, p in outs[1:]:
        assert same(u, outs[0][0]) and same(p, outs[0][1])
    oracle.set_sphere_form(True)
    try:
        u_p, psi_p = oracle.ic2d_passive_sums(vx, fx, zf, fa, fm, eps)
    finally:
        oracle.set_sphere_form(False)
    assert rel(outs[0][0].cpu(), u_p) < TOL32
    assert rel(outs[0][1].cpu(), psi_p) < TOL32
    for bad in (6, -2):
        with pytest.raises(core.LpmError, match="0-5"):
            ctx.set_kernel_shape(bad)


def test_argument_errors(gpu_ctx):
    ctx = gpu_ctx
    L = core.lib()
    nullv = core.View(None, 0, 0)
    rc = L.lpm_bve_vertex_velocity(ctx.handle, nullv, nullv, 10, nullv, None, None, None, 10)
    assert rc == core.LPM_ERR_ARG
    assert b"null" in L.lpm_last_error()
    rc = L.lpm_context_set_precision(ctx.handle, 16)
    assert rc == core.LPM_ERR_ARG
    with pytest.raises(core.LpmError):
        core.check(L.lpm_ic2d_passive_sums(ctx.handle, 4, nullv, None, nullv, 0, nullv, None, None,
                                           None, 0.0, 0))


def test_tendencies_and_invariants(gpu_ctx, oracle):
    ctx = gpu_ctx
    vx, fx, fa, fm, zf = sphere_case(3)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((fx.shape[0], 3))
    dz = torch.zeros(fx.shape[0], dtype=torch.float64, device="cuda")
    F.bve_vorticity_tendency(ctx, dz, dev(u), 0.01, OMEGA)
    ctx.synchronize()
    assert np.array_equal(dz.cpu().numpy(), -2.0 * OMEGA * u[:, 2] * 0.01)
    F.ic2d_tendencies(ctx, dz, dev(u), OMEGA)
    ctx.synchronize()
    assert np.array_equal(dz.cpu().numpy(), -(2 * OMEGA * u[:, 2]))
    inv = F.ic2d_invariants(ctx, dev(zf), dev(u), dev(fa), dev(fm))
    ref = oracle.invariants(zf, u, fa, fm)
    # sums in a different order: compare against the sum of magnitudes
    leaf = fm == 0
    scale = [np.abs(zf * fa)[leaf].sum(), 0.5 * (zf * zf * fa)[leaf].sum(),
             0.5 * ((u * u).sum(1) * fa)[leaf].sum()]
    for a, b, s in zip(inv, ref, scale):
        assert abs(a - b) <= 1e-13 * s
    tg = torch.zeros(fx.shape[0], dtype=torch.float64, device="cuda")
    F.sphere_tangency(ctx, tg, dev(fx), dev(u))
    ctx.synchronize()
    assert np.array_equal(tg.cpu().numpy(),
                          (fx[:, 0] * u[:, 0] + fx[:, 1] * u[:, 1]) + fx[:, 2] * u[:, 2])
    en = F.err_norms(ctx, dev(u + 1e-3), dev(u), dev(fa), dev(fm))
    er = oracle.err_norms(u + 1e-3, u, fa, fm)
    assert np.allclose(en, er, rtol=1e-12)


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_one_call_direct_sums(gpu_ctx, precision):
    """lpm_bve_direct_sum / lpm_plane_direct_sum (per-thread context, caller's
    stream) give the context-based functors' results bit for bit."""
    import ctypes as C

    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F
    from lpm_gb300.core import check, crd3, lib, ptr

    prec = getattr(core, precision)
    ctx = core.Context(0, precision=prec)
    d = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=d)
    for kind, ndim in ((core.MESH_ICOS_TRI, 3), (core.MESH_QUAD_RECT, 2)):
        vx, fx, fa, fm = core.build_mesh(kind, 4, 1.0)
        z = np.sin(2 * fx[:, 0]) + fx[:, 1]
        T = {k: torch.tensor(v, device=d) for k, v in dict(vx=vx, fx=fx, fa=fa, fm=fm, z=z).items()}
        fn = lib().lpm_bve_direct_sum if ndim == 3 else lib().lpm_plane_direct_sum
        for eps in (0.0, 0.02):
            for coll in (0, 1):
                if ndim == 2 and eps == 0.0 and not coll:
                    continue
                tgt = T["fx"] if coll else T["vx"]
                n = tgt.shape[0]
                u1 = torch.zeros(n, ndim, dtype=torch.float64, device=d)
                p1 = torch.zeros(n, dtype=torch.float64, device=d)
                with torch.cuda.stream(stream):
                    check(fn(crd3(tgt), crd3(T["fx"]), ptr(T["z"]), ptr(T["fa"]), ptr(T["fm"]),
                             fx.shape[0], coll, eps, 3, prec, ptr(u1), ndim, 1, ptr(p1),
                             C.c_void_p(stream.cuda_stream)))
                stream.synchronize()
                u2 = torch.zeros_like(u1)
                p2 = torch.zeros_like(p1)
                if ndim == 3 and eps == 0.0:
                    if coll:
                        F.bve_face_solve(ctx, p2, u2, T["fx"], T["z"], T["fa"], T["fm"])
                    else:
                        F.bve_vertex_solve(ctx, p2, u2, T["vx"], T["fx"], T["z"], T["fa"], T["fm"])
                elif coll:
                    F.ic2d_active_sums(ctx, u2, p2, T["fx"], T["z"], T["fa"], T["fm"], eps,
                                       self_rule=1 if ndim == 3 else 0)
                else:
                    F.ic2d_passive_sums(ctx, u2, p2, T["vx"], T["fx"], T["z"], T["fa"], T["fm"], eps)
                torch.cuda.synchronize()
                # parent slots coincide with a child: non-finite in both
                for a, b in ((u1, u2), (p1, p2)):
                    fa_, fb_ = torch.isfinite(a), torch.isfinite(b)
                    assert torch.equal(fa_, fb_), (kind, eps, coll)
                    assert torch.equal(a[fa_], b[fb_]), (kind, eps, coll)
    # releasing the thread's cached context frees it; the next call makes a new one
    check(lib().lpm_one_call_release())
    u3 = torch.zeros_like(u1)
    p3 = torch.zeros_like(p1)
    with torch.cuda.stream(stream):
        check(fn(crd3(tgt), crd3(T["fx"]), ptr(T["z"]), ptr(T["fa"]), ptr(T["fm"]), fx.shape[0],
                 coll, eps, 3, prec, ptr(u3), ndim, 1, ptr(p3), C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    assert torch.equal(u3, u1) and torch.equal(p3, p1)
    check(lib().lpm_one_call_release())


@pytest.mark.parametrize("level", [4, 5])
@pytest.mark.parametrize("eps", [0.0, 0.01])
def test_fp64_hoisted_vs_exact(gpu_ctx, level, eps):
    """LPM_FP64 (hoisted cross product, Newton-Raphson quotients) against
    LPM_FP64_EXACT (the reference's term-by-term arithmetic) on vertices and
    leaf faces: within 1e-12, and the two share their inputs exactly."""
    ctx = gpu_ctx
    vx, fx, fa, fm, zf = sphere_case(level, noise=0.5)
    T = [dev(a) for a in (vx, fx, zf, fa, fm)]
    out = {}
    for prec in (core.FP64, core.FP64_EXACT):
        ctx.set_precision(prec)
        vu = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
        vp = torch.zeros(vx.shape[0], dtype=torch.float64, device="cuda")
        fu = torch.zeros(fx.shape[0], 3, dtype=torch.float64, device="cuda")
        fp = torch.zeros(fx.shape[0], dtype=torch.float64, device="cuda")
        if eps == 0.0:
            F.bve_vertex_solve(ctx, vp, vu, T[0], T[1], T[2], T[3], T[4])
            F.bve_face_solve(ctx, fp, fu, T[1], T[2], T[3], T[4])
        else:
            F.ic2d_passive_sums(ctx, vu, vp, T[0], T[1], T[2], T[3], T[4], eps)
            F.ic2d_active_sums(ctx, fu, fp, T[1], T[2], T[3], T[4], eps, self_rule=1)
        ctx.synchronize()
        out[prec] = [a.cpu().numpy() for a in (vu, vp, fu, fp)]
    leaf = fm == 0
    a, b = out[core.FP64], out[core.FP64_EXACT]
    assert rel(a[0], b[0]) < TOL64 and rel(a[1], b[1]) < TOL64
    assert rel(a[2][leaf], b[2][leaf]) < TOL64 and rel(a[3][leaf], b[3][leaf]) < TOL64

"""Planar SWE direct sums on the GPU against the FP64 oracle: vertex sums and
face sums (collocated i == j skip for eps = 0), every output, masked parent
slots excluded, FP64 parity 1e-12 (ErrNorms linf normalisation per output)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ["u", "du1dx1", "du1dx2", "du2dx1", "du2dx2", "laps", "psi", "phi"]


def _fields(level):
    from lpm_gb300 import core

    vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, level, 4.0)
    zeta = 2 * np.exp(-np.sum((fx - [1.0, 0.0]) ** 2, 1)) - 2 * np.exp(-np.sum((fx + [1.0, 0.0]) ** 2, 1))
    sigma = 0.3 * np.cos(fx[:, 0]) * np.exp(-np.sum(fx ** 2, 1) / 8)
    fs = 1 + 0.1 * np.exp(-np.sum(fx ** 2, 1))
    vs = 1 + 0.1 * np.exp(-np.sum(vx ** 2, 1))
    return vx, fx, fa, fm, zeta, sigma, fs, vs


def _check(got, ref9):
    cols = {"u": ref9[:, 0:2], "du1dx1": ref9[:, 2], "du1dx2": ref9[:, 3], "du2dx1": ref9[:, 4],
            "du2dx2": ref9[:, 5], "laps": ref9[:, 6], "psi": ref9[:, 7], "phi": ref9[:, 8]}
    for k in KEYS:
        g = got[k].cpu().numpy()
        r = cols[k]
        err = np.max(np.abs(g - r)) / max(np.max(np.abs(r)), 1e-300)
        assert err < 1e-12, (k, err)
    dd = ref9[:, 2] ** 2 + 2 * ref9[:, 3] * ref9[:, 4] + ref9[:, 5] ** 2
    g = got["ddot"].cpu().numpy()
    assert np.max(np.abs(g - dd)) / np.max(np.abs(dd)) < 1e-12


@pytest.mark.parametrize("eps", [0.0, 0.05])
def test_swe_plane_parity(gpu_ctx, oracle, eps):
    import torch

    from lpm_gb300 import functors as F

    vx, fx, fa, fm, zeta, sigma, fs, vs = _fields(5)
    h = math.sqrt(fa[fm == 0].mean())
    pse_eps = h ** 0.55  # PSEKernel::get_epsilon(dx, 11/20)
    d = torch.device("cuda", gpu_ctx.device)
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, sg=sigma, fs=fs, vs=vs).items()}
    gv = F.swe_plane_vertex_sums(gpu_ctx, T["vx"], T["vs"], T["fx"], T["z"], T["sg"], T["fa"],
                                 T["fm"], T["fs"], eps, pse_eps)
    gf = F.swe_plane_face_sums(gpu_ctx, T["fx"], T["z"], T["sg"], T["fa"], T["fm"], T["fs"], eps,
                               pse_eps)
    torch.cuda.synchronize()
    rv = oracle.swe_plane_sums(vx, vs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps, collocated=False)
    rf = oracle.swe_plane_sums(fx, fs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps,
                               collocated=not eps > 0)
    _check(gv, rv)
    _check(gf, rf)


def test_swe_do_velocity_false_keeps_u(gpu_ctx):
    import torch

    from lpm_gb300 import core
    from lpm_gb300.core import check, lib, ptr, view

    vx, fx, fa, fm, zeta, sigma, fs, vs = _fields(3)
    d = torch.device("cuda", gpu_ctx.device)
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(fx=fx, fa=fa, fm=fm, z=zeta, sg=sigma, fs=fs).items()}
    u = torch.full((fx.shape[0], 2), 7.0, dtype=torch.float64, device=d)
    outs = [torch.zeros(fx.shape[0], dtype=torch.float64, device=d) for _ in range(8)]
    check(lib().lpm_swe_plane_face_sums(gpu_ctx.handle, view(u), *(ptr(o) for o in outs),
                                        view(T["fx"]), ptr(T["z"]), ptr(T["sg"]), ptr(T["fa"]),
                                        ptr(T["fm"]), ptr(T["fs"]), fx.shape[0], 0.05, 0.3, 0))
    torch.cuda.synchronize()
    assert bool((u == 7.0).all())
    with pytest.raises(core.LpmError):
        check(lib().lpm_swe_plane_face_sums(gpu_ctx.handle, view(u), *(ptr(o) for o in outs),
                                            view(T["fx"]), ptr(T["z"]), ptr(T["sg"]), ptr(T["fa"]),
                                            ptr(T["fm"]), ptr(T["fs"]), fx.shape[0], 0.05, 0.0, 1))


# ---- spherical SWE sums ------------------------------------------------------

def _sphere_fields(level, seed=5):
    from lpm_gb300 import core

    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, level, 1.0)
    rng = np.random.default_rng(seed)
    zeta = 2 * fx[:, 2] + np.sin(3 * fx[:, 0]) + 0.1 * rng.standard_normal(fx.shape[0])
    sigma = np.cos(2 * fx[:, 2]) * fx[:, 1] + 0.1 * rng.standard_normal(fx.shape[0])
    return vx, fx, fa, fm, zeta, sigma


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _dev(gpu_ctx, **arrays):
    import torch

    d = torch.device("cuda", gpu_ctx.device)
    return {k: torch.tensor(v, device=d) for k, v in arrays.items()}


@pytest.mark.parametrize("eps,tag", [(0.0, "e0"), (0.05, "e5")])
def test_swe_sphere_golden(gpu_ctx, oracle, eps, tag):
    """Against the reference's pair polynomials in extended precision
    (tests/golden/swe_sphere_icos_l3.npz)."""
    import torch
    from pathlib import Path

    from lpm_gb300 import functors as F

    g = np.load(Path(__file__).resolve().parent / "golden" / "swe_sphere_icos_l3.npz")
    T = _dev(gpu_ctx, vx=g["vx"], fx=g["fx"], fa=g["fa"], fm=g["fm"], z=g["zeta"], s=g["sigma"])
    gv = F.swe_sphere_vertex_sums(gpu_ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                  want_grad=True)
    gf = F.swe_sphere_face_sums(gpu_ctx, T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                want_grad=True)
    torch.cuda.synchronize()
    ft = g["face_targets"]
    for o, ref, sel in ((gv, g[f"vert_{tag}"], slice(None)), (gf, g[f"face_{tag}"], ft)):
        u = o["u"].cpu().numpy()[sel]
        m = o["grad"].cpu().numpy()[sel]
        dd = o["ddot"].cpu().numpy()[sel]
        assert _rel(u, ref[:, :3]) < 1e-13
        assert _rel(m, ref[:, 3:]) < 1e-12
        assert _rel(dd, oracle.double_dot(ref[:, 3:])) < 1e-12


@pytest.mark.parametrize("eps", [0.0, 0.02])
def test_swe_sphere_parity(gpu_ctx, oracle, eps):
    """Icosahedral level 5 vertices and level 4 faces (all slots, masked
    parents excluded as sources) against the FP64 oracle."""
    import torch

    from lpm_gb300 import functors as F

    vx, fx, fa, fm, zeta, sigma = _sphere_fields(5)
    T = _dev(gpu_ctx, vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma)
    gv = F.swe_sphere_vertex_sums(gpu_ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                  want_grad=True)
    torch.cuda.synchronize()
    rv = oracle.swe_sphere_sums(vx, fx, zeta, sigma, fa, fm, eps)
    assert _rel(gv["u"].cpu().numpy(), rv[:, :3]) < 1e-12
    assert _rel(gv["grad"].cpu().numpy(), rv[:, 3:]) < 1e-12
    assert _rel(gv["ddot"].cpu().numpy(), oracle.double_dot(rv[:, 3:])) < 1e-12
    vx, fx, fa, fm, zeta, sigma = _sphere_fields(4)
    T = _dev(gpu_ctx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma)
    gf = F.swe_sphere_face_sums(gpu_ctx, T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                want_grad=True)
    torch.cuda.synchronize()
    rf = oracle.swe_sphere_sums(fx, fx, zeta, sigma, fa, fm, eps, collocated=eps == 0)
    leaf = fm == 0  # a parent slot coincides with its central child: 1/0 there
    got_u = gf["u"].cpu().numpy()
    assert np.array_equal(np.isfinite(got_u), np.isfinite(rf[:, :3]))
    assert _rel(got_u[leaf], rf[leaf, :3]) < 1e-12
    assert _rel(gf["grad"].cpu().numpy()[leaf], rf[leaf, 3:]) < 1e-12
    assert _rel(gf["ddot"].cpu().numpy()[leaf], oracle.double_dot(rf[leaf, 3:])) < 1e-12


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_swe_sphere_views_and_flags(oracle, precision):
    """LayoutLeft-style strided views, do_velocity = 0 keeps u, no grad
    pointer, all sources masked, zero targets, argument errors."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F
    from lpm_gb300.core import check, lib, ptr, view

    gpu_ctx = core.Context(0, precision=getattr(core, precision))
    vx, fx, fa, fm, zeta, sigma = _sphere_fields(3)
    T = _dev(gpu_ctx, vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma)
    ref = F.swe_sphere_vertex_sums(gpu_ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"],
                                   0.01)
    # SoA with component stride nmax > n
    def soa(a, extra=13):
        buf = torch.zeros(3, a.shape[0] + extra, dtype=torch.float64, device=a.device)
        buf[:, :a.shape[0]] = a.T
        return buf[:, :a.shape[0]].T
    vxs, fxs = soa(T["vx"]), soa(T["fx"])
    us = soa(torch.zeros_like(T["vx"]))
    o = {"u": us, "ddot": torch.zeros(vx.shape[0], dtype=torch.float64, device=us.device)}
    F.swe_sphere_vertex_sums(gpu_ctx, vxs, fxs, T["z"], T["s"], T["fa"], T["fm"], 0.01, out=o)
    torch.cuda.synchronize()
    assert torch.equal(o["u"], ref["u"]) and torch.equal(o["ddot"], ref["ddot"])
    # do_velocity = 0 leaves u alone, still writes ddot
    o = {"u": torch.full_like(T["vx"], 7.0),
         "ddot": torch.zeros(vx.shape[0], dtype=torch.float64, device=us.device)}
    F.swe_sphere_vertex_sums(gpu_ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"], 0.01,
                             do_velocity=False, out=o)
    torch.cuda.synchronize()
    assert bool((o["u"] == 7.0).all()) and torch.equal(o["ddot"], ref["ddot"])
    # every source masked: zeros
    allm = torch.ones_like(T["fm"])
    z = F.swe_sphere_face_sums(gpu_ctx, T["fx"], T["z"], T["s"], T["fa"], allm, 0.01)
    torch.cuda.synchronize()
    assert not bool(z["u"].any()) and not bool(z["ddot"].any())
    # zero targets is a no-op
    check(lib().lpm_swe_sphere_vertex_sums(gpu_ctx.handle, view(T["vx"]), ptr(o["ddot"]), None,
                                           view(T["vx"]), 0, view(T["fx"]), ptr(T["z"]),
                                           ptr(T["s"]), ptr(T["fa"]), ptr(T["fm"]), fx.shape[0],
                                           0.0, 1))
    with pytest.raises(core.LpmError):
        check(lib().lpm_swe_sphere_face_sums(gpu_ctx.handle, view(T["fx"]), ptr(o["ddot"]), None,
                                             view(T["fx"]), ptr(T["z"]), ptr(T["s"]), ptr(T["fa"]),
                                             ptr(T["fm"]), fx.shape[0], -1.0, 1))


@pytest.mark.parametrize("eps", [0.0, 0.02])
def test_swe_sphere_fp32c(oracle, eps):
    """FP32-compensated form (chord moments, hi/lo positions) against the FP64
    oracle: velocity within 1e-6, gradient tensor and double dot product
    within 2e-5 (relative to the largest value), leaf targets."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F

    ctx = core.Context(0, precision=core.FP32C)
    vx, fx, fa, fm, zeta, sigma = _sphere_fields(5)
    T = _dev(ctx, vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma)
    gv = F.swe_sphere_vertex_sums(ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                  want_grad=True)
    torch.cuda.synchronize()
    rv = oracle.swe_sphere_sums(vx, fx, zeta, sigma, fa, fm, eps)
    errs = [_rel(gv["u"].cpu().numpy(), rv[:, :3]), _rel(gv["grad"].cpu().numpy(), rv[:, 3:]),
            _rel(gv["ddot"].cpu().numpy(), oracle.double_dot(rv[:, 3:]))]
    vx, fx, fa, fm, zeta, sigma = _sphere_fields(4)
    T = _dev(ctx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma)
    gf = F.swe_sphere_face_sums(ctx, T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                want_grad=True)
    torch.cuda.synchronize()
    rf = oracle.swe_sphere_sums(fx, fx, zeta, sigma, fa, fm, eps, collocated=eps == 0)
    leaf = fm == 0
    errs += [_rel(gf["u"].cpu().numpy()[leaf], rf[leaf, :3]),
             _rel(gf["grad"].cpu().numpy()[leaf], rf[leaf, 3:]),
             _rel(gf["ddot"].cpu().numpy()[leaf], oracle.double_dot(rf[leaf, 3:]))]
    print("fp32c errors (vertex u, M, ddot; face u, M, ddot):", ["%.2e" % e for e in errs])
    assert errs[0] < 1e-6 and errs[3] < 1e-6
    assert max(errs[1], errs[2], errs[4], errs[5]) < 2e-5


@pytest.mark.parametrize("eps", [0.0, 0.05])
def test_swe_plane_fp32c(oracle, eps):
    """Planar FP32-compensated form (moments, hi/lo positions and surface)
    against the FP64 oracle: velocity within 1e-6, stream and potential
    functions within 3e-6 (the MUFU log2 carries ~2e-7 absolute error per
    pair), gradients, double dot and PSE Laplacian within 3e-5."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F

    ctx = core.Context(0, precision=core.FP32C)
    vx, fx, fa, fm, zeta, sigma, fs, vs = _fields(5)
    pse_eps = math.sqrt(fa[fm == 0].mean()) ** 0.55
    d = torch.device("cuda", 0)
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, sg=sigma, fs=fs, vs=vs).items()}
    gv = F.swe_plane_vertex_sums(ctx, T["vx"], T["vs"], T["fx"], T["z"], T["sg"], T["fa"],
                                 T["fm"], T["fs"], eps, pse_eps)
    gf = F.swe_plane_face_sums(ctx, T["fx"], T["z"], T["sg"], T["fa"], T["fm"], T["fs"], eps,
                               pse_eps)
    torch.cuda.synchronize()
    rv = oracle.swe_plane_sums(vx, vs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps, collocated=False)
    rf = oracle.swe_plane_sums(fx, fs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps,
                               collocated=not eps > 0)
    tol = {"u": 1e-6, "psi": 3e-6, "phi": 3e-6, "du1dx1": 3e-5, "du1dx2": 3e-5, "du2dx1": 3e-5,
           "du2dx2": 3e-5, "laps": 3e-5}
    leaf = fm == 0
    worst = {}
    for got, ref, sel in ((gv, rv, slice(None)), (gf, rf, leaf)):
        cols = {"u": ref[:, 0:2], "du1dx1": ref[:, 2], "du1dx2": ref[:, 3], "du2dx1": ref[:, 4],
                "du2dx2": ref[:, 5], "laps": ref[:, 6], "psi": ref[:, 7], "phi": ref[:, 8]}
        for k, t in tol.items():
            e = _rel(got[k].cpu().numpy()[sel], cols[k][sel])
            worst[k] = max(worst.get(k, 0.0), e)
            assert e < t, (k, e)
        dd = ref[:, 2] ** 2 + 2 * ref[:, 3] * ref[:, 4] + ref[:, 5] ** 2
        assert _rel(got["ddot"].cpu().numpy()[sel], dd[sel]) < 3e-5
    print("plane fp32c errors:", {k: "%.1e" % v for k, v in worst.items()})


def test_swe_plane_fp32c_views_and_flags():
    """Planar FP32C form: LayoutLeft-style views give the same bits as AoS,
    do_velocity = 0 keeps u, all sources masked give zeros."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F

    ctx = core.Context(0, precision=core.FP32C)
    vx, fx, fa, fm, zeta, sigma, fs, vs = _fields(3)
    d = torch.device("cuda", 0)
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, sg=sigma, fs=fs, vs=vs).items()}
    ref = F.swe_plane_vertex_sums(ctx, T["vx"], T["vs"], T["fx"], T["z"], T["sg"], T["fa"],
                                  T["fm"], T["fs"], 0.05, 0.3)

    def soa(a, extra=7):
        buf = torch.zeros(a.shape[1], a.shape[0] + extra, dtype=torch.float64, device=a.device)
        buf[:, :a.shape[0]] = a.T
        return buf[:, :a.shape[0]].T
    got = F.swe_plane_vertex_sums(ctx, soa(T["vx"]), T["vs"], soa(T["fx"]), T["z"], T["sg"],
                                  T["fa"], T["fm"], T["fs"], 0.05, 0.3)
    torch.cuda.synchronize()
    for k in ("u", "ddot", "laps", "psi", "phi"):
        assert torch.equal(got[k], ref[k]), k
    z = F.swe_plane_face_sums(ctx, T["fx"], T["z"], T["sg"], T["fa"], torch.ones_like(T["fm"]),
                              T["fs"], 0.05, 0.3)
    torch.cuda.synchronize()
    assert not bool(z["u"].any()) and not bool(z["psi"].any())


@pytest.mark.parametrize("eps", [0.0, 0.05])
def test_swe_fp32c_odd_source_count(oracle, eps):
    """The FP32C kernels take their sources two at a time; with an odd count
    the last pair carries a zero-strength dummy at the origin.  One leaf more
    is masked here so the count is odd, and the quad mesh has a vertex at the
    origin (with eps = 0 the dummy coincides with that target): both forms
    stay within their tolerances of the FP64 oracle."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F

    ctx = core.Context(0, precision=core.FP32C)
    d = torch.device("cuda", 0)
    # plane
    vx, fx, fa, fm, zeta, sigma, fs, vs = _fields(4)
    fm = fm.copy()
    fm[np.flatnonzero(fm == 0)[7]] = 1
    assert (fm == 0).sum() % 2 == 1 and np.any(np.all(vx == 0, axis=1))
    pse_eps = math.sqrt(fa[fm == 0].mean()) ** 0.55
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, sg=sigma, fs=fs, vs=vs).items()}
    gv = F.swe_plane_vertex_sums(ctx, T["vx"], T["vs"], T["fx"], T["z"], T["sg"], T["fa"],
                                 T["fm"], T["fs"], eps, pse_eps)
    gf = F.swe_plane_face_sums(ctx, T["fx"], T["z"], T["sg"], T["fa"], T["fm"], T["fs"], eps,
                               pse_eps)
    torch.cuda.synchronize()
    rv = oracle.swe_plane_sums(vx, vs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps, collocated=False)
    rf = oracle.swe_plane_sums(fx, fs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps,
                               collocated=not eps > 0)
    tol = {"u": 1e-6, "psi": 3e-6, "phi": 3e-6, "du1dx1": 3e-5, "du1dx2": 3e-5, "du2dx1": 3e-5,
           "du2dx2": 3e-5, "laps": 3e-5}
    leaf = fm == 0
    for got, ref, sel in ((gv, rv, slice(None)), (gf, rf, leaf)):
        cols = {"u": ref[:, 0:2], "du1dx1": ref[:, 2], "du1dx2": ref[:, 3], "du2dx1": ref[:, 4],
                "du2dx2": ref[:, 5], "laps": ref[:, 6], "psi": ref[:, 7], "phi": ref[:, 8]}
        for k, t in tol.items():
            g = got[k].cpu().numpy()[sel]
            assert np.isfinite(g).all(), k
            assert _rel(g, cols[k][sel]) < t, k
    # sphere
    vx, fx, fa, fm, zeta, sigma = _sphere_fields(4)
    fm = fm.copy()
    fm[np.flatnonzero(fm == 0)[7]] = 1
    assert (fm == 0).sum() % 2 == 1
    T = _dev(ctx, vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma)
    gv = F.swe_sphere_vertex_sums(ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                  want_grad=True)
    gf = F.swe_sphere_face_sums(ctx, T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                want_grad=True)
    torch.cuda.synchronize()
    rv = oracle.swe_sphere_sums(vx, fx, zeta, sigma, fa, fm, eps)
    rf = oracle.swe_sphere_sums(fx, fx, zeta, sigma, fa, fm, eps, collocated=eps == 0)
    leaf = fm == 0
    for got, ref, sel in ((gv, rv, slice(None)), (gf, rf, leaf)):
        assert _rel(got["u"].cpu().numpy()[sel], ref[sel, :3]) < 1e-6
        assert _rel(got["grad"].cpu().numpy()[sel], ref[sel, 3:]) < 2e-5

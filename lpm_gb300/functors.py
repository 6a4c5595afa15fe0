"""One call per reference Kokkos functor launch on the direct-sum path.

Each function takes device tensors (torch, on the context's GPU) with the
reference functor's argument meaning and launches the matching CUDA path:

=========================  =====================================================
function                   reference (pbosler/lpm)
=========================  =====================================================
bve_vertex_solve           BVEVertexSolve   src/lpm_bve_sphere_kernels.hpp:90
bve_vertex_stream_fn       BVEVertexStreamFn                          :141
bve_vertex_velocity        BVEVertexVelocity                          :179
bve_face_solve             BVEFaceSolve                               :284
bve_face_stream_fn         BVEFaceStreamFn                            :329
bve_face_velocity          BVEFaceVelocity                            :365
bve_vorticity_tendency     BVEVorticityTendency                       :399
ic2d_passive_sums          Incompressible2DPassiveSums  src/lpm_incompressible2d_kernels.hpp:144
ic2d_active_sums           Incompressible2DActiveSums                 :201
ic2d_tendencies            Incompressible2DTendencies                 :257
=========================  =====================================================

``nsrc`` / ``n_active`` is the number of face slots (all tree levels); the
mask excludes divided faces.  Arithmetic follows ``ctx.precision``.
"""
from __future__ import annotations

from .core import check, lib, ptr, view, View


def _n(t):
    return 0 if t is None else int(t.shape[0])


def bve_vertex_solve(ctx, psi, u, vx, fx, zeta, area, mask, nsrc=None):
    nsrc = _n(fx) if nsrc is None else nsrc
    check(lib().lpm_bve_vertex_solve(ctx.handle, ptr(psi), view(u), view(vx), _n(vx), view(fx),
                                     ptr(zeta), ptr(area), ptr(mask), nsrc))


def bve_vertex_stream_fn(ctx, psi, vx, fx, zeta, area, mask, nsrc=None):
    nsrc = _n(fx) if nsrc is None else nsrc
    check(lib().lpm_bve_vertex_stream_fn(ctx.handle, ptr(psi), view(vx), _n(vx), view(fx),
                                         ptr(zeta), ptr(area), ptr(mask), nsrc))


def bve_vertex_velocity(ctx, u, vx, fx, zeta, area, mask, nsrc=None):
    nsrc = _n(fx) if nsrc is None else nsrc
    check(lib().lpm_bve_vertex_velocity(ctx.handle, view(u), view(vx), _n(vx), view(fx),
                                        ptr(zeta), ptr(area), ptr(mask), nsrc))


def bve_face_solve(ctx, psi, u, fx, zeta, area, mask, nsrc=None):
    nsrc = _n(fx) if nsrc is None else nsrc
    check(lib().lpm_bve_face_solve(ctx.handle, ptr(psi), view(u), view(fx), ptr(zeta),
                                   ptr(area), ptr(mask), nsrc))


def bve_face_stream_fn(ctx, psi, fx, zeta, area, mask, nsrc=None):
    nsrc = _n(fx) if nsrc is None else nsrc
    check(lib().lpm_bve_face_stream_fn(ctx.handle, ptr(psi), view(fx), ptr(zeta), ptr(area),
                                       ptr(mask), nsrc))


def bve_face_velocity(ctx, u, fx, zeta, area, mask, nsrc=None):
    nsrc = _n(fx) if nsrc is None else nsrc
    check(lib().lpm_bve_face_velocity(ctx.handle, view(u), view(fx), ptr(zeta), ptr(area),
                                      ptr(mask), nsrc))


def bve_vorticity_tendency(ctx, dzeta, u, dt, Omega):
    check(lib().lpm_bve_vorticity_tendency(ctx.handle, ptr(dzeta), view(u), _n(u), dt, Omega))


def ic2d_passive_sums(ctx, u, psi, x, y, zeta, area, mask, eps, n_active=None):
    ndim = int(x.shape[1])
    n_active = _n(y) if n_active is None else n_active
    check(lib().lpm_ic2d_passive_sums(ctx.handle, ndim, view(u), ptr(psi), view(x), _n(x),
                                      view(y), ptr(zeta), ptr(area), ptr(mask), eps, n_active))


def ic2d_active_sums(ctx, u, psi, xy, zeta, area, mask, eps, n_active=None, self_rule=0):
    ndim = int(xy.shape[1])
    n_active = _n(xy) if n_active is None else n_active
    check(lib().lpm_ic2d_active_sums(ctx.handle, ndim, view(u), ptr(psi), view(xy), ptr(zeta),
                                     ptr(area), ptr(mask), eps, n_active, self_rule))


def ic2d_tendencies(ctx, dzeta, u, cor):
    check(lib().lpm_ic2d_tendencies(ctx.handle, int(u.shape[1]), ptr(dzeta), view(u), _n(u), cor))


def sphere_tangency(ctx, udotx, x, u):
    """SphereTangentFunctor (src/lpm_sphere_functions.hpp:59-78): x . u per point."""
    check(lib().lpm_sphere_tangency(ctx.handle, ptr(udotx), view(x), view(u), _n(x)))


_SWE_KEYS = ("ddot", "du1dx1", "du1dx2", "du2dx1", "du2dx2", "laps", "psi", "phi")


def _swe_outputs(n, like):
    import torch

    out = {k: torch.zeros(n, dtype=torch.float64, device=like.device) for k in _SWE_KEYS}
    out["u"] = torch.zeros(n, 2, dtype=torch.float64, device=like.device)
    return out


def swe_plane_vertex_sums(ctx, vx, vs, fx, fzeta, fsigma, farea, fmask, fs, eps, pse_eps,
                          do_velocity=True):
    """PlanarSWEVertexSums (src/lpm_swe_kernels.hpp:626-721): dict of outputs."""
    o = _swe_outputs(_n(vx), vx)
    check(lib().lpm_swe_plane_vertex_sums(
        ctx.handle, view(o["u"]), *(ptr(o[k]) for k in _SWE_KEYS), view(vx), ptr(vs), _n(vx),
        view(fx), ptr(fzeta), ptr(fsigma), ptr(farea), ptr(fmask), ptr(fs), _n(fx), eps, pse_eps,
        int(do_velocity)))
    return o


def swe_plane_face_sums(ctx, fx, fzeta, fsigma, farea, fmask, fs, eps, pse_eps, do_velocity=True):
    """PlanarSWEFaceSums (src/lpm_swe_kernels.hpp:787-876): dict of outputs."""
    o = _swe_outputs(_n(fx), fx)
    check(lib().lpm_swe_plane_face_sums(
        ctx.handle, view(o["u"]), *(ptr(o[k]) for k in _SWE_KEYS), view(fx), ptr(fzeta),
        ptr(fsigma), ptr(farea), ptr(fmask), ptr(fs), _n(fx), eps, pse_eps, int(do_velocity)))
    return o


def _sphere_swe_outputs(n, like, want_grad):
    import torch

    out = {"u": torch.zeros(n, 3, dtype=torch.float64, device=like.device),
           "ddot": torch.zeros(n, dtype=torch.float64, device=like.device)}
    if want_grad:
        out["grad"] = torch.zeros(n, 9, dtype=torch.float64, device=like.device)
    return out


def swe_sphere_vertex_sums(ctx, vx, fx, fzeta, fsigma, farea, fmask, eps, do_velocity=True,
                           want_grad=False, out=None):
    """SphereVertexSums (src/lpm_swe_kernels.hpp:723-785): dict with u (n x 3),
    ddot (n) and, if want_grad, the summed gradient tensor (n x 9, row-major).
    `out` reuses a dict from an earlier call (u keeps its values when
    do_velocity is false)."""
    o = out if out is not None else _sphere_swe_outputs(_n(vx), vx, want_grad)
    check(lib().lpm_swe_sphere_vertex_sums(
        ctx.handle, view(o["u"]), ptr(o["ddot"]), ptr(o.get("grad")), view(vx), _n(vx), view(fx),
        ptr(fzeta), ptr(fsigma), ptr(farea), ptr(fmask), _n(fx), eps, int(do_velocity)))
    return o


def swe_sphere_face_sums(ctx, fx, fzeta, fsigma, farea, fmask, eps, do_velocity=True,
                         want_grad=False, out=None):
    """SphereFaceSums (src/lpm_swe_kernels.hpp:877-940): as swe_sphere_vertex_sums
    at every face slot (i == j skipped for |eps| < DBL_EPSILON)."""
    o = out if out is not None else _sphere_swe_outputs(_n(fx), fx, want_grad)
    check(lib().lpm_swe_sphere_face_sums(
        ctx.handle, view(o["u"]), ptr(o["ddot"]), ptr(o.get("grad")), view(fx), ptr(fzeta),
        ptr(fsigma), ptr(farea), ptr(fmask), _n(fx), eps, int(do_velocity)))
    return o


def ic2d_invariants(ctx, zeta, vel, area, mask):
    import ctypes as C
    out = (C.c_double * 3)()
    check(lib().lpm_ic2d_invariants(ctx.handle, int(vel.shape[1]), _n(zeta), ptr(zeta), view(vel),
                                    ptr(area), ptr(mask), out))
    return tuple(out)


def err_norms(ctx, appx, exact, wt=None, mask=None):
    """ErrNorms (src/lpm_error.hpp:81-91): (l1, l2, linf)."""
    import ctypes as C
    out = (C.c_double * 3)()
    a = appx if appx.dim() == 2 else appx.reshape(-1, 1)
    e = exact if exact.dim() == 2 else exact.reshape(-1, 1)
    check(lib().lpm_err_norms(ctx.handle, int(a.shape[1]), _n(a), view(a), view(e), ptr(wt),
                              ptr(mask), out))
    return tuple(out)


__all__ = [n for n in dir() if not n.startswith("_") and n not in ("check", "lib", "ptr", "view", "View")]

"""Incompressible2D / Incompressible2DRK2 with the reference's method names.

Mirrors ``Incompressible2D<SeedType>`` (src/lpm_incompressible2d.hpp,
src/lpm_incompressible2d_impl.hpp) and ``Incompressible2DRK2``
(src/lpm_incompressible2d_rk2.hpp, _impl.hpp:15-172) for the sphere
(CoriolisSphere) and the plane (CoriolisBetaPlane).
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import functors as F
from .core import (FP64, MESH_QUAD_RECT, build_mesh, check, default_context, eval_ic, lib, ptr,
                   view)


class Incompressible2D:
    """Particles, mesh and fields of 2D incompressible flow.

    ``coriolis``: Omega of CoriolisSphere (default 2 pi) or (f0, beta) of
    CoriolisBetaPlane (default (0, 0)).
    """

    def __init__(self, seed: int, level: int, radius: float = 1.0, eps: float = 0.0,
                 coriolis=None, ctx=None, device: int = 0):
        self.ctx = ctx if ctx is not None else default_context(device)
        self.dev = torch.device("cuda", self.ctx.device)
        vx, fx, fa, fm = build_mesh(seed, level, radius)
        self.ndim = vx.shape[1]
        self.sphere = self.ndim == 3
        if coriolis is None:
            coriolis = 2 * math.pi if self.sphere else (0.0, 0.0)
        self.coriolis = coriolis
        self.host_face_mask = fm
        dev = self.dev
        self.vert_x = torch.from_numpy(vx).to(dev)
        self.face_x = torch.from_numpy(fx).to(dev)
        self.face_area = torch.from_numpy(fa).to(dev)
        self.face_mask = torch.from_numpy(fm).to(dev)
        nv, nf, nd = vx.shape[0], fx.shape[0], self.ndim
        z = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
        self.rel_vort_passive, self.rel_vort_active = z(nv), z(nf)
        self.abs_vort_passive, self.abs_vort_active = z(nv), z(nf)
        self.stream_fn_passive, self.stream_fn_active = z(nv), z(nf)
        self.velocity_passive, self.velocity_active = z(nv, nd), z(nf, nd)
        self.eps = float(eps)
        self.t = 0.0

    @property
    def cor_param(self) -> float:
        """Omega (sphere) or beta (plane): what dfdt multiplies."""
        return float(self.coriolis) if self.sphere else float(self.coriolis[1])

    def _f(self, xh):
        if self.sphere:
            return 2 * float(self.coriolis) * xh[:, 2]
        f0, beta = self.coriolis
        return f0 + beta * xh[:, 1]

    def n_vertices_host(self) -> int:
        return int(self.vert_x.shape[0])

    def n_faces_host(self) -> int:
        return int(self.face_x.shape[0])

    def init_vorticity(self, kind: int, params=()) -> None:
        """src/lpm_incompressible2d_impl.hpp:139-173."""
        for x, rel, ab in ((self.vert_x, self.rel_vort_passive, self.abs_vort_passive),
                           (self.face_x, self.rel_vort_active, self.abs_vort_active)):
            xh = x.cpu().numpy()
            zeta = eval_ic(kind, params, xh)
            rel.copy_(torch.from_numpy(zeta))
            ab.copy_(torch.from_numpy(zeta + self._f(xh)))

    def init_direct_sums(self, self_rule: int = 0) -> None:
        """Passive + active sums (src/lpm_incompressible2d_impl.hpp:235-254)."""
        F.ic2d_passive_sums(self.ctx, self.velocity_passive, self.stream_fn_passive, self.vert_x,
                            self.face_x, self.rel_vort_active, self.face_area, self.face_mask,
                            self.eps)
        F.ic2d_active_sums(self.ctx, self.velocity_active, self.stream_fn_active, self.face_x,
                           self.rel_vort_active, self.face_area, self.face_mask, self.eps,
                           self_rule=self_rule)

    def advance_timestep(self, solver: "Incompressible2DRK2") -> None:
        solver.advance_timestep_impl()
        self.t = solver.t_idx * solver.dt

    def total_vorticity(self) -> float:
        return F.ic2d_invariants(self.ctx, self.rel_vort_active, self.velocity_active,
                                 self.face_area, self.face_mask)[0]

    def total_enstrophy(self) -> float:
        return F.ic2d_invariants(self.ctx, self.rel_vort_active, self.velocity_active,
                                 self.face_area, self.face_mask)[1]

    def total_kinetic_energy(self) -> float:
        return F.ic2d_invariants(self.ctx, self.rel_vort_active, self.velocity_active,
                                 self.face_area, self.face_mask)[2]


class Incompressible2DRK2:
    """Heun RK2 (src/lpm_incompressible2d_rk2_impl.hpp:74-172)."""

    def __init__(self, dt: float, ic2d: Incompressible2D, precision: int = FP64, flags: int = 0):
        self.dt = float(dt)
        self.ic2d = ic2d
        self.t_idx = 0
        self.n_passive = ic2d.n_vertices_host()
        self.n_active = ic2d.n_faces_host()
        self.eps = ic2d.eps
        self._h = C.c_void_p()
        check(lib().lpm_ic2d_rk2_create(ic2d.ctx.handle, C.byref(self._h), ic2d.ndim,
                                        self.n_passive, self.n_active, self.dt, self.eps,
                                        ic2d.cor_param, precision, int(flags)))

    def advance_timestep_impl(self) -> None:
        s = self.ic2d
        check(lib().lpm_ic2d_rk2_advance_timestep(
            self._h, view(s.vert_x), ptr(s.rel_vort_passive), view(s.velocity_passive),
            ptr(s.stream_fn_passive), view(s.face_x), ptr(s.rel_vort_active),
            view(s.velocity_active), ptr(s.stream_fn_active), ptr(s.face_area),
            ptr(s.face_mask)))
        self.t_idx += 1

    def nbody_time(self) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_int64()
        check(lib().lpm_ic2d_rk2_nbody_time(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def close(self) -> None:
        if self._h:
            lib().lpm_ic2d_rk2_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def colliding_dipoles_params(strength=2.0, radius=1.0, x0=2.0):
    """CollidingDipolePairPlane(+s, r, (-x0, 0), -s, r, (+x0, 0))."""
    return (strength, radius, -x0, 0.0, -strength, radius, x0, 0.0)


__all__ = ["Incompressible2D", "Incompressible2DRK2", "colliding_dipoles_params",
           "MESH_QUAD_RECT"]

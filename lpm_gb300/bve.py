"""BVESphere / BVERK4 with the reference's method names, on the CUDA path.

Mirrors ``BVESphere<SeedType>`` (src/lpm_bve_sphere.hpp:24-109,
src/lpm_bve_sphere_impl.hpp) and ``BVERK4`` (src/lpm_bve_rk4.hpp:10-77).
Fields are device tensors (torch, float64) laid out like the reference's
views: coordinates and vectors n x 3 (LayoutRight), scalars n.  Divided
(parent) faces keep their slots with mask = 1 and area = 0, as in the
reference's face arrays.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import functors as F
from .core import (FP64, IC_GAUSSIAN_SPHERE, IC_RH54, IC_SOLID_BODY, MESH_ICOS_TRI,
                   build_mesh, check, default_context, eval_ic, lib, ptr, view)

TWO_PI = 2 * math.pi


class BVESphere:
    """Meshed particles of the barotropic vorticity equation on the sphere.

    ``BVESphere(nmaxverts, nmaxedges, nmaxfaces)`` + ``tree_init(depth, seed)``
    of the reference collapse into ``BVESphere(level, seed)`` here.
    """

    def __init__(self, level: int, seed: int = MESH_ICOS_TRI, ctx=None, device: int = 0):
        self.ctx = ctx if ctx is not None else default_context(device)
        self.dev = torch.device("cuda", self.ctx.device)
        vx, fx, fa, fm = build_mesh(seed, level, 1.0)
        self.host_vert_x, self.host_face_x, self.host_face_area, self.host_face_mask = vx, fx, fa, fm
        dev = self.dev
        self.vert_x = torch.from_numpy(vx).to(dev)
        self.face_x = torch.from_numpy(fx).to(dev)
        self.face_area = torch.from_numpy(fa).to(dev)
        self.face_mask = torch.from_numpy(fm).to(dev)
        nv, nf = vx.shape[0], fx.shape[0]
        z = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
        self.rel_vort_verts, self.abs_vort_verts, self.stream_fn_verts = z(nv), z(nv), z(nv)
        self.velocity_verts = z(nv, 3)
        self.rel_vort_faces, self.abs_vort_faces, self.stream_fn_faces = z(nf), z(nf), z(nf)
        self.velocity_faces = z(nf, 3)
        self.Omega = TWO_PI  # src/lpm_bve_sphere_impl.hpp:27
        self._omg_set = False
        self.t = 0.0

    # ---- checkpoint / restart ------------------------------------------
    # The reference has no restart for this path; the state of a run is the
    # particle arrays below plus Omega and t (the steppers keep nothing
    # between steps), so a snapshot of them resumes a run bit for bit.
    _STATE = ("vert_x", "rel_vort_verts", "abs_vort_verts", "stream_fn_verts", "velocity_verts",
              "face_x", "rel_vort_faces", "abs_vort_faces", "stream_fn_faces", "velocity_faces",
              "face_area", "face_mask")

    def save(self, path) -> None:
        """Writes the particle state, Omega and t to an .npz file."""
        arrays = {k: getattr(self, k).cpu().numpy() for k in self._STATE}
        np.savez(path, Omega=self.Omega, t=self.t, omega_set=self._omg_set,
                 host_vert_x=self.host_vert_x, host_face_x=self.host_face_x, **arrays)

    @classmethod
    def from_snapshot(cls, path, ctx=None, device: int = 0) -> "BVESphere":
        """A BVESphere holding the state written by save()."""
        self = cls.__new__(cls)
        self.ctx = ctx if ctx is not None else default_context(device)
        self.dev = torch.device("cuda", self.ctx.device)
        with np.load(path) as z:
            for k in self._STATE:
                setattr(self, k, torch.from_numpy(z[k]).to(self.dev))
            self.host_vert_x, self.host_face_x = z["host_vert_x"], z["host_face_x"]
            self.host_face_area, self.host_face_mask = z["face_area"], z["face_mask"]
            self.Omega, self.t = float(z["Omega"]), float(z["t"])
            self._omg_set = bool(z["omega_set"])
        return self

    def n_vertices_host(self) -> int:
        return int(self.vert_x.shape[0])

    def n_faces_host(self) -> int:
        return int(self.face_x.shape[0])

    def n_leaves(self) -> int:
        return int((self.host_face_mask == 0).sum())

    def set_omega(self, omg: float) -> None:
        if not self._omg_set:
            self.Omega = float(omg)
            self._omg_set = True

    def init_vorticity(self, kind: int, params=()) -> None:
        """rel_vort = f(x); abs_vort = f + 2 Omega z (src/lpm_bve_sphere_impl.hpp:148-179)."""
        for x_dev, xh, rel, ab in ((self.vert_x, None, self.rel_vort_verts, self.abs_vort_verts),
                                   (self.face_x, None, self.rel_vort_faces, self.abs_vort_faces)):
            xh = x_dev.cpu().numpy()
            zeta = eval_ic(kind, params, xh)
            rel.copy_(torch.from_numpy(zeta))
            ab.copy_(torch.from_numpy(zeta + 2 * self.Omega * xh[:, 2]))

    def init_velocity(self) -> None:
        """BVEVertexVelocity + BVEFaceVelocity (src/lpm_bve_sphere_impl.hpp:181-205)."""
        F.bve_vertex_velocity(self.ctx, self.velocity_verts, self.vert_x, self.face_x,
                              self.rel_vort_faces, self.face_area, self.face_mask)
        F.bve_face_velocity(self.ctx, self.velocity_faces, self.face_x, self.rel_vort_faces,
                            self.face_area, self.face_mask)

    def init_stream_fn(self) -> None:
        """BVEVertexStreamFn + BVEFaceStreamFn (src/lpm_bve_sphere_impl.hpp:207-231)."""
        F.bve_vertex_stream_fn(self.ctx, self.stream_fn_verts, self.vert_x, self.face_x,
                               self.rel_vort_faces, self.face_area, self.face_mask)
        F.bve_face_stream_fn(self.ctx, self.stream_fn_faces, self.face_x, self.rel_vort_faces,
                             self.face_area, self.face_mask)


class BVERK4:
    """Classic RK4 for BVESphere (src/lpm_bve_rk4_impl.hpp:55-167).

    ``precision``: FP64 (reference arithmetic) or FP32C.  ``eps`` > 0 uses the
    smoothed sphere kernel 1 - x.y + eps^2 of Incompressible2DKernels.
    ``flags``: core.STEP_* options (quirk fix, reprojection, masked targets).
    """

    def __init__(self, dt: float, sph: BVESphere, precision: int = FP64, eps: float = 0.0,
                 flags: int = 0):
        self.dt = float(dt)
        self.Omega = sph.Omega
        self.nverts = sph.n_vertices_host()
        self.nfaces = sph.n_faces_host()
        self.precision, self.eps, self.flags = precision, float(eps), int(flags)
        self.ctx = sph.ctx
        self._h = C.c_void_p()
        check(lib().lpm_bve_rk4_create(self.ctx.handle, C.byref(self._h), self.nverts,
                                       self.nfaces, self.dt, self.Omega, self.eps,
                                       precision, self.flags))

    def advance_timestep(self, sph: BVESphere) -> None:
        check(lib().lpm_bve_rk4_advance_timestep(
            self._h, view(sph.vert_x), ptr(sph.rel_vort_verts), view(sph.velocity_verts),
            view(sph.face_x), ptr(sph.rel_vort_faces), view(sph.velocity_faces),
            ptr(sph.face_area), ptr(sph.face_mask)))
        sph.t += self.dt

    def set_farfield(self, ff, rebuild_every: int = 0) -> None:
        """Evaluate the stages with an octree far field (FP64_CHORD steppers)."""
        check(lib().lpm_bve_rk4_set_farfield(self._h, ff.handle if ff is not None else None,
                                             int(rebuild_every)))
        self._ff = ff  # keep it alive as long as the stepper

    def nbody_time(self) -> tuple[float, int]:
        """(ms, launches) of the N-body kernels timed since the last call
        (requires core.STEP_TIME_NBODY)."""
        ms, n = C.c_double(), C.c_int64()
        check(lib().lpm_bve_rk4_nbody_time(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def kernel_shape(self) -> tuple[int, int, int]:
        """(threads per CTA, targets per thread, CTAs per SM of the register
        cap) of the N-body kernel this stepper runs; after the first step."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(lib().lpm_bve_rk4_kernel_shape(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def close(self) -> None:
        if self._h:
            lib().lpm_bve_rk4_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rossby_haurwitz_params(Omega: float = TWO_PI) -> tuple[float, float]:
    """RH R=4 with omega = K = Omega/12.5: RossbyHaurwitz54(u0=omega, amp=-K)."""
    w = Omega / 12.5
    return (w, -w)


def gaussian_params(strength=4 * math.pi, b=4.0, lon=0.0, lat=math.pi / 20, gauss_const=0.0,
                    background_Omega=0.0):
    return (strength, b, lon, lat, gauss_const, background_Omega)


__all__ = ["BVESphere", "BVERK4", "rossby_haurwitz_params", "gaussian_params",
           "IC_GAUSSIAN_SPHERE", "IC_RH54", "IC_SOLID_BODY"]

"""Ensembles of independent BVE sphere problems advanced together.

``BVEEnsemble`` holds many ``BVESphere``-like problems back to back in one set
of device arrays and advances them with one persistent N-body launch per
evaluation (C ABI ``lpm_ensemble_*``).  Each problem has the reference's
BVERK4 semantics; only the chord-form velocity (FP32C / FP64_CHORD) is
available here.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from .core import (FP32C, IC_MULTI_GAUSSIAN, MESH_ICOS_TRI, build_mesh, check, default_context,
                   eval_ic, lib, ptr, view)


def random_vortex_params(rng: np.random.Generator, kmin=1, kmax=4, amp=(math.pi, 4 * math.pi),
                         width=(0.1, 0.4)):
    """1-4 Gaussian vortices with centres uniform on the sphere, amplitudes
    and widths uniform in the given ranges: MULTI_GAUSSIAN parameters."""
    k = int(rng.integers(kmin, kmax + 1))
    prm = [float(k)]
    for _ in range(k):
        z = rng.uniform(-1, 1)
        lon = rng.uniform(0, 2 * math.pi)
        lat = math.asin(z)
        a = rng.uniform(*amp)
        w = rng.uniform(*width)
        prm += [a, 1.0 / w, lon, lat]  # exp(-(1 - x.c)/w^2) = exp(-b^2 (1 - x.c)), b = 1/w
    return prm


class BVEEnsemble:
    def __init__(self, levels, params, dt, eps=0.0, Omega=2 * math.pi, precision=FP32C,
                 flags=0, ctx=None, device=0):
        self.ctx = ctx if ctx is not None else default_context(device)
        dev = torch.device("cuda", self.ctx.device)
        vxs, fxs, fas, fms, vzs, fzs = [], [], [], [], [], []
        for lev, prm in zip(levels, params):
            vx, fx, fa, fm = build_mesh(MESH_ICOS_TRI, int(lev), 1.0)
            vxs.append(vx)
            fxs.append(fx)
            fas.append(fa)
            fms.append(fm)
            vzs.append(eval_ic(IC_MULTI_GAUSSIAN, prm, vx))
            fzs.append(eval_ic(IC_MULTI_GAUSSIAN, prm, fx))
        self.nverts = np.array([v.shape[0] for v in vxs], np.int64)
        self.nfaces = np.array([f.shape[0] for f in fxs], np.int64)
        self.nleaves = np.array([int((m == 0).sum()) for m in fms], np.int64)
        cat = lambda xs: torch.from_numpy(np.ascontiguousarray(np.concatenate(xs))).to(dev)
        self.vx, self.fx = cat(vxs), cat(fxs)
        self.vzeta, self.fzeta = cat(vzs), cat(fzs)
        self.farea, self.fmask = cat(fas), cat(fms)
        self.vvel = torch.zeros_like(self.vx)
        self.fvel = torch.zeros_like(self.fx)
        self.dt, self.eps, self.precision = float(dt), float(eps), precision
        self._h = C.c_void_p()
        check(lib().lpm_ensemble_create(self.ctx.handle, C.byref(self._h), len(levels),
                                        self.nverts.ctypes.data, self.nfaces.ctypes.data,
                                        ptr(self.fmask), self.dt, Omega, self.eps, precision,
                                        int(flags)))

    def interactions_per_evaluation(self) -> int:
        return int(((self.nverts + self.nleaves) * self.nleaves).sum())

    def velocity(self):
        check(lib().lpm_ensemble_velocity(self._h, view(self.vx), view(self.vvel), view(self.fx),
                                          ptr(self.fzeta), view(self.fvel), ptr(self.farea)))

    def advance_timestep(self):
        check(lib().lpm_ensemble_advance_timestep(self._h, view(self.vx), ptr(self.vzeta),
                                                  view(self.vvel), view(self.fx),
                                                  ptr(self.fzeta), view(self.fvel),
                                                  ptr(self.farea)))

    def info(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().lpm_ensemble_info(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"chunk_len": a.value, "items": b.value, "targets": c.value}

    def shape(self):
        """(threads per CTA, targets per thread, persistent) of the N-body
        kernel in use."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(lib().lpm_ensemble_shape(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, bool(c.value)

    def set_kernel(self, shape: int, persistent: bool):
        """Fixes the kernel shape (index 0-5) and launch form (before the
        first evaluation, together with set_chunk_len)."""
        check(lib().lpm_ensemble_set_kernel(self._h, int(shape), int(bool(persistent))))

    def set_chunk_len(self, n: int):
        check(lib().lpm_ensemble_set_chunk_len(self._h, int(n)))

    def nbody_time(self):
        ms, n = C.c_double(), C.c_int64()
        check(lib().lpm_ensemble_nbody_time(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def problem_slices(self, p):
        v0 = int(self.nverts[:p].sum())
        f0 = int(self.nfaces[:p].sum())
        return slice(v0, v0 + int(self.nverts[p])), slice(f0, f0 + int(self.nfaces[p]))

    def close(self):
        if self._h:
            lib().lpm_ensemble_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

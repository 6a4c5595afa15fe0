"""Octree far field with a learned correction (no reference counterpart).

``FarField`` wraps ``lpm_farfield_*``: an octree over the face sources
(leaves <= ``leaf_max`` points), target blocks of 128 Morton-ordered targets,
the order-4 Cartesian expansion of the chord-form sphere kernel for accepted
cells (h <= theta (D - r_block)), the exact FP32-compensated sum over the
near leaves, and -- once trained or loaded -- a BF16 MLP run on the tcgen05
tensor cores that predicts the expansion's residual for accepted cells with
h / (D - r_block) >= rho_min.  The exact direct sum stays the fallback (a
target block whose lists overflow) and the reference for its error (tests, bench).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .core import check, default_context, lib, ptr, view

NPARAM = 40960
NNORM = 97
NIN = 48


class FarField:
    def __init__(self, theta: float = 0.5, leaf_max: int = 64, rho_min: float = 0.25,
                 ctx=None, device: int = 0):
        self.ctx = ctx if ctx is not None else default_context(device)
        self.theta, self.leaf_max, self.rho_min = float(theta), int(leaf_max), float(rho_min)
        self._h = C.c_void_p()
        check(lib().lpm_farfield_create(self.ctx.handle, C.byref(self._h), self.theta,
                                        self.leaf_max, self.rho_min))

    @property
    def handle(self):
        return self._h

    def velocity(self, u, x, fx, zeta, area, mask, eps: float) -> None:
        """BVE sphere velocity at targets x (torch, device) from face slots."""
        check(lib().lpm_farfield_velocity(self._h, view(u), view(x), int(x.shape[0]), view(fx),
                                          ptr(zeta), ptr(area), ptr(mask), int(fx.shape[0]),
                                          float(eps)))

    def train(self, nsamples: int = 1 << 24, epochs: int = 8, batch: int = 16384,
              lr: float = 2e-3, seed: int = 20261203, level_min: int = 5, level_max: int = 8,
              eps: float = 0.01) -> list[float]:
        """Trains on the GPU; returns the mean loss of every epoch."""
        loss = (C.c_float * epochs)()
        check(lib().lpm_farfield_train(self._h, int(nsamples), int(epochs), int(batch), float(lr),
                                       C.c_uint64(int(seed)), int(level_min), int(level_max),
                                       float(eps), loss))
        return list(loss)

    def set_network(self, enable: bool) -> None:
        check(lib().lpm_farfield_set_network(self._h, int(bool(enable))))

    def get_weights(self) -> tuple[np.ndarray, np.ndarray]:
        w = np.zeros(NPARAM, np.float32)
        n = np.zeros(NNORM, np.float32)
        check(lib().lpm_farfield_get_weights(self._h, w.ctypes.data, n.ctypes.data))
        return w, n

    def set_weights(self, w: np.ndarray, norm: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.float32)
        norm = np.ascontiguousarray(norm, np.float32)
        if w.size != NPARAM or norm.size != NNORM:
            raise ValueError("weights must hold 40960 floats and the normalisation 97")
        check(lib().lpm_farfield_set_weights(self._h, w.ctypes.data, norm.ctypes.data))

    def grad(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        """Gradient of the mean squared error from the tensor-core training
        kernel for rows x (n x 48, normalised inputs) and targets y (n x 3)."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(NPARAM, np.float32)
        check(lib().lpm_farfield_grad(self._h, x.ctypes.data, y.ctypes.data, int(x.shape[0]),
                                      g.ctypes.data))
        return g

    def stats(self) -> dict:
        out = (C.c_int64 * 7)()
        check(lib().lpm_farfield_stats(self._h, out))
        return {"far_pairs": out[0], "near_pairs_x128": out[1], "learned_pairs": out[2],
                "fallback_blocks": out[3], "cells": out[4], "target_blocks": out[5],
                "network_rows": out[6]}

    def timing(self, enable: bool) -> tuple[float, float, int]:
        """(tree ms, network ms, evaluations) since the last call; then
        enables or disables event timing of the following evaluations."""
        a, b, n = C.c_double(), C.c_double(), C.c_int64()
        check(lib().lpm_farfield_timing(self._h, int(bool(enable)), C.byref(a), C.byref(b),
                                        C.byref(n)))
        return a.value, b.value, n.value

    def close(self) -> None:
        if self._h:
            lib().lpm_farfield_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def octree_stats(src_xyz: np.ndarray, tgt_xyz: np.ndarray, leaf_max: int = 64) -> dict:
    """Host-only summary of the octree and target blocks (no GPU needed)."""
    s = np.ascontiguousarray(src_xyz, np.float64)
    t = np.ascontiguousarray(tgt_xyz, np.float64)
    out = np.zeros(9, np.int64)
    check(lib().lpm_octree_stats(s.ctypes.data, s.shape[0], t.ctypes.data if t.size else None,
                                 t.shape[0], int(leaf_max), out.ctypes.data))
    keys = ["cells", "leaves", "max_leaf", "max_level", "blocks", "min_block_fill",
            "targets_covered", "sources_in_leaves", "errors"]
    return dict(zip(keys, (int(v) for v in out)))


def tc_selftest(ctx, A, B, N: int, K: int, a_mn: bool, b_mn: bool):
    """D = A B on the tensor cores (see lpm_tc_selftest); torch float32 on the device."""
    import torch
    D = torch.zeros(128, N, dtype=torch.float32, device=A.device)
    check(lib().lpm_tc_selftest(ctx.handle, ptr(A), ptr(B), ptr(D), int(N), int(K), int(a_mn),
                                int(b_mn)))
    return D


def split_weights(w: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Master vector -> W1 (128x48), W2, W3 (128x128), W4 (16x128)."""
    w = np.asarray(w)
    a, b, c = 128 * 48, 128 * 48 + 128 * 128, 128 * 48 + 2 * 128 * 128
    return (w[:a].reshape(128, 48), w[a:b].reshape(128, 128), w[b:c].reshape(128, 128),
            w[c:].reshape(16, 128))


__all__ = ["FarField", "octree_stats", "tc_selftest", "split_weights", "NPARAM", "NNORM", "NIN"]

"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the octree far field's
per-cell mathematics (lpm_gb300/csrc/ffmath.cuh, farfield.cu, mlp.cu):
cell records, the order-4 Cartesian expansion of the chord-form sphere
kernel, the learned correction's input features and its training target.
Imported by tests only; never by the product path.

Kernel: u(x) = -(1/2pi) sum_j g_j (x cross y_j) / (|x - y_j|^2 + c0),
c0 = 2 eps^2, which equals the reference's biot_savart with the smoothing
1 - x.y + eps^2 for unit vectors (src/lpm_sphere_functions.hpp:44-57,
src/lpm_incompressible2d_kernels.hpp:35-47).
"""
from __future__ import annotations

import math

import numpy as np


def monomials(p=4):
    """Exponents (a, b, c) of degree <= p: by degree, then a, then b descending."""
    out = []
    for n in range(p + 1):
        for a in range(n, -1, -1):
            for b in range(n - a, -1, -1):
                out.append((a, b, n - a - b))
    return out


MON = monomials(4)
IDX = {m: i for i, m in enumerate(MON)}


def cell_frame(c):
    n = c / np.linalg.norm(c)
    r = np.array([0.0, 0.0, 1.0]) if abs(n[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    e1 = np.cross(r, n)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(n, e1)
    return np.stack([e1, e2, n])


def complex_index():
    """(p, q, k, part) of the 35 real complex-moment features, part 0 = Re, 1 = Im."""
    out = []
    for k in range(5):
        for n in range(5 - k):
            for p in range(n, (n + 1) // 2 - 1, -1):
                q = n - p
                if p > q:
                    out += [(p, q, k, 0), (p, q, k, 1)]
                else:
                    out += [(p, q, k, 0)]
    return out


CIDX = complex_index()


def cell_record(y, g):
    """Centre (mean of the points), radius, frame and moments of one cell."""
    y = np.asarray(y, np.float64)
    g = np.asarray(g, np.float64)
    c = y.mean(axis=0)
    Q = cell_frame(c)
    d = (y - c) @ Q.T
    h = float(np.max(np.linalg.norm(d, axis=1)))
    S = float(np.abs(g).sum())
    M = np.array([np.sum(g * d[:, 0] ** a * d[:, 1] ** b * d[:, 2] ** k) for a, b, k in MON])
    z = d[:, 0] + 1j * d[:, 1]
    C = []
    for p, q, k, part in CIDX:
        v = np.sum(g * z ** p * np.conj(z) ** q * d[:, 2] ** k) / (S * h ** (p + q + k))
        C.append(v.real if part == 0 else v.imag)
    return {"c": c, "Q": Q, "h": h, "S": S, "M": M, "C": np.array(C), "n": len(g)}


def exact(y, g, x, c0):
    """Chord-form velocity of the points (y, g) at targets x."""
    d = x[:, None, :] - y[None, :, :]
    q = np.sum(d * d, axis=2) + c0
    w = np.einsum("ij,ijk->ik", g[None, :] / q, d)
    return -np.cross(w, x) / (2 * math.pi)


def expansion(cell, x, c0):
    """Order-4 expansion about the centre: u = -(1/2pi) x cross (c S + V)/R^2
    with the Chebyshev-U recurrence of 1/q in delta."""
    Q, c, M = cell["Q"], cell["c"], cell["M"]
    d = (x - c) @ Q.T
    R2 = np.sum(d * d, axis=1) + c0
    a = d / R2[:, None]
    s = 1.0 / R2
    # polynomials P_n(delta) as {monomial: coefficient array}
    P = [{(0, 0, 0): np.ones(len(x))}]

    def mul_lin(poly):
        out = {}
        for (i, j, k), v in poly.items():
            for ax in range(3):
                m = [i, j, k]
                m[ax] += 1
                m = tuple(m)
                out[m] = out.get(m, 0) + v * a[:, ax]
        return out

    def mul_r2(poly):
        out = {}
        for (i, j, k), v in poly.items():
            for ax in range(3):
                m = [i, j, k]
                m[ax] += 2
                m = tuple(m)
                out[m] = out.get(m, 0) + v
        return out

    P.append({m: 2 * v for m, v in mul_lin(P[0]).items()})
    for n in range(2, 5):
        A, B = mul_lin(P[n - 1]), mul_r2(P[n - 2])
        nxt = {m: 2 * v for m, v in A.items()}
        for m, v in B.items():
            nxt[m] = nxt.get(m, 0) - s * v
        P.append(nxt)
    S = np.zeros(len(x))
    V = np.zeros((len(x), 3))
    for n in range(5):
        for m, v in P[n].items():
            S += v * M[IDX[m]]
            if n <= 3:
                for ax in range(3):
                    mm = list(m)
                    mm[ax] += 1
                    V[:, ax] += v * M[IDX[tuple(mm)]]
    W = (V + np.outer(S, [0.0, 0.0, np.linalg.norm(c)])) * s[:, None]
    Wg = W @ Q  # back to the global frame
    return -np.cross(x, Wg) / (2 * math.pi)


def canonical(cell, x):
    """Per-target rotation about the cell normal (cs, sn), distance D, rho,
    tangential and normal offsets."""
    d = (x - cell["c"]) @ cell["Q"].T
    dt = np.hypot(d[:, 0], d[:, 1])
    D = np.linalg.norm(d, axis=1)
    cs = np.where(dt > 0, d[:, 0] / np.where(dt > 0, dt, 1), 1.0)
    sn = np.where(dt > 0, d[:, 1] / np.where(dt > 0, dt, 1), 0.0)
    return cs, sn, D, cell["h"] / D, dt, d[:, 2]


def features(cell, x, eps):
    """Raw network inputs (n x 48): rotated complex moments, dt/D, dn/D, rho,
    eps/D, h, the constant 1 at index 40, zeros after."""
    cs, sn, D, rho, dt, dn = canonical(cell, x)
    phase = (cs + 1j * sn)
    f = np.zeros((len(x), 48))
    j = 0
    Cv = cell["C"]
    while j < 35:
        p, q, k, part = CIDX[j]
        m = p - q
        if m > 0:
            z = (Cv[j] + 1j * Cv[j + 1]) * phase ** (-m)
            f[:, j], f[:, j + 1] = z.real, z.imag
            j += 2
        else:
            f[:, j] = Cv[j]
            j += 1
    f[:, 35] = dt / D
    f[:, 36] = dn / D
    f[:, 37] = rho
    f[:, 38] = eps / D
    f[:, 39] = cell["h"]
    f[:, 40] = 1.0
    return f


def residual_target(cell, y, g, x, c0):
    """Exact minus expansion velocity in the target's canonical frame,
    divided by S rho^5 / (2 pi D): the network's training target."""
    R = exact(y, g, x, c0) - expansion(cell, x, c0)
    cs, sn, D, rho, _, _ = canonical(cell, x)
    e1, e2, n = cell["Q"]
    E1 = cs[:, None] * e1 + sn[:, None] * e2
    E2 = -sn[:, None] * e1 + cs[:, None] * e2
    scale = cell["S"] * rho ** 5 / (2 * math.pi * D)
    return np.stack([np.sum(R * E1, 1), np.sum(R * E2, 1), R @ n], 1) / scale[:, None]


def correction(cell, x, out, out_scale):
    """Network output (n x 3, normalised) -> velocity correction (global)."""
    cs, sn, D, rho, _, _ = canonical(cell, x)
    scale = out_scale * cell["S"] * rho ** 5 / (2 * math.pi * D)
    r = out[:, :3] * scale[:, None]
    e1, e2, n = cell["Q"]
    v1 = r[:, 0] * cs - r[:, 1] * sn
    v2 = r[:, 0] * sn + r[:, 1] * cs
    R = v1[:, None] * e1 + v2[:, None] * e2 + r[:, 2:3] * n
    return R - x * np.sum(x * R, 1)[:, None]

"""CPU pins of the algebra behind the FP32C SWE kernels (k_swe_sphere32,
k_swe_plane32 in lpm_gb300/csrc/swe.cu): the per-target moment sums and the
epilogue that assembles velocity, gradient tensor, Laplacian and potentials
from them, restated here in FP64 numpy, reproduce the reference's pair sums.

Sphere: against tests/golden/swe_sphere_icos_l3.npz (the reference's own
gradient polynomials in extended precision).  Plane: against the FP64
oracle (oracle_swe_plane_sums, the reference's operation order)."""
import math
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "swe_sphere_icos_l3.npz"


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _xmat(v):
    return np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])


def sphere_moment_form(tx, y, zeta, sigma, area, mask, eps, tgt_idx=None):
    """(n x 12): u and M from the chord moments of d = x - y."""
    keep = mask == 0
    out = []
    e2 = eps * eps
    for n, x in enumerate(tx):
        k = keep.copy()
        if tgt_idx is not None:
            k[tgt_idx[n]] = False
        d = x - y[k]
        rs = -zeta[k] * area[k] / (2 * math.pi)
        ps = -sigma[k] * area[k] / (2 * math.pi)
        dd = np.sum(d * d, 1)
        r = 1.0 / (dd + 2 * e2)
        sz, ss = rs * r, ps * r
        R, Q = 2 * sz * r, 2 * ss * r
        A, B = sz @ d, ss @ d
        U1, V1 = R @ d, Q @ d
        U2 = np.einsum("j,ja,jb->ab", R, d, d)
        V2 = np.einsum("j,ja,jb->ab", Q, d, d)
        Z, G, H = sz.sum(), ss.sum(), ss @ dd
        P = np.eye(3) - np.outer(x, x)
        u = np.cross(A, x) - P @ B
        T1 = np.stack([np.cross(U2[:, b], x) for b in range(3)], axis=1)
        M = (e2 * np.outer(np.cross(U1, x), x) + T1 + e2 * np.outer(x, P @ V1) + V2 @ P
             + _xmat(Z * x - A) - (G - 0.5 * H) * P)
        out.append(np.concatenate([u, M.ravel()]))
    return np.array(out)


@pytest.mark.parametrize("eps,tag", [(0.0, "e0"), (0.05, "e5")])
def test_sphere_moment_form_matches_reference_polynomials(eps, tag):
    g = np.load(GOLD)
    v = sphere_moment_form(g["vx"], g["fx"], g["zeta"], g["sigma"], g["fa"], g["fm"], eps)
    ft = g["face_targets"]
    f = sphere_moment_form(g["fx"][ft], g["fx"], g["zeta"], g["sigma"], g["fa"], g["fm"], eps,
                           tgt_idx=ft if eps == 0 else None)
    for got, ref in ((v, g[f"vert_{tag}"]), (f, g[f"face_{tag}"])):
        assert _rel(got[:, :3], ref[:, :3]) < 1e-13
        assert _rel(got[:, 3:], ref[:, 3:]) < 1e-12


def plane_moment_form(tx, ts, y, zeta, sigma, area, mask, sfc, eps, pse_eps):
    """(n x 9): u, v, the four gradients, lap(s), psi, phi from 15 moments."""
    keep = mask == 0
    out = []
    for x, sx in zip(tx, ts):
        d = x - y[keep]
        rot, pot = (zeta * area)[keep], (sigma * area)[keep]
        dd = np.sum(d * d, 1)
        Rr = dd + eps * eps
        r = 1.0 / Rr
        a, b = rot * r, pot * r
        a2, b2 = a * r, b * r
        w = [a @ d[:, 0], a @ d[:, 1], b @ d[:, 0], b @ d[:, 1], a.sum(), b.sum(),
             a2 @ (d[:, 0] ** 2), a2 @ (d[:, 0] * d[:, 1]), a2 @ (d[:, 1] ** 2),
             b2 @ (d[:, 0] ** 2), b2 @ (d[:, 0] * d[:, 1]), b2 @ (d[:, 1] ** 2)]
        p2 = dd / (pse_eps * pse_eps)
        poly = ((-2.0 / 3.0 * p2 + 10.0) * p2 - 40.0) * p2 + 40.0
        lap = ((sfc[keep] - sx) * area[keep]) @ (poly * np.exp(-p2))
        L = np.log2(Rr)
        pi = math.pi
        out.append([(w[2] - w[1]) / (2 * pi), (w[0] + w[3]) / (2 * pi),
                    (w[7] - w[9]) / pi + w[5] / (2 * pi), (w[8] - w[10]) / pi - w[4] / (2 * pi),
                    -(w[6] + w[10]) / pi + w[4] / (2 * pi), -(w[7] + w[11]) / pi + w[5] / (2 * pi),
                    lap / (pi * pse_eps * pse_eps),
                    -math.log(2) / (4 * pi) * (rot @ L), -math.log(2) / (4 * pi) * (pot @ L)])
    return np.array(out)


def test_plane_moment_form_matches_oracle(oracle):
    import lpm_oracle as O

    vx, fx, fa, fm = O.mesh(O.MESH_QUAD_RECT, 3, 4.0)
    zeta = 2 * np.exp(-np.sum((fx - [1.0, 0.0]) ** 2, 1)) - 2 * np.exp(-np.sum((fx + [1.0, 0.0]) ** 2, 1))
    sigma = 0.3 * np.cos(fx[:, 0]) * np.exp(-np.sum(fx ** 2, 1) / 8)
    fs = 1 + 0.1 * np.exp(-np.sum(fx ** 2, 1))
    vs = 1 + 0.1 * np.exp(-np.sum(vx ** 2, 1))
    got = plane_moment_form(vx, vs, fx, zeta, sigma, fa, fm, fs, 0.05, 0.3)
    ref = oracle.swe_plane_sums(vx, vs, fx, zeta, sigma, fa, fm, fs, 0.05, 0.3)
    for c in range(9):
        assert _rel(got[:, c], ref[:, c]) < 1e-12, c

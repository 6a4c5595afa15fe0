"""Generates tests/golden/swe_sphere_icos_l3.npz: the reference's spherical SWE
pair formulas (src/lpm_swe_kernels.hpp: kzeta_sphere :63-76, ksigma_sphere
:87-108, grad_kzeta :114-150, grad_ksigma :179-325, summed as in
SphereSweDirectSumReducer :608-619) evaluated in extended precision on FP64
inputs.

    python tests/golden/make_swe_sphere_golden.py [path/to/lpm_swe_kernels.hpp]

The velocity-gradient entries are not restated: the script reads the
reference header as text, turns each `gkz[k] = ...;` / `gks[k] = ...;`
expression into a numpy expression and evaluates it with np.longdouble
(64-bit significand on x86-64), so the fixture holds the reference's own
polynomials to ~1e-18 relative per pair.  The FP64 oracle and the CUDA path,
which evaluate equivalent compact forms, are pinned against these values.
"""
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from lpm_gb300 import core  # noqa: E402

LD = np.longdouble
PI = LD("3.14159265358979323846264338327950288")


def read_polynomials(header: Path):
    text = header.read_text()
    out = {}
    for name in ("gkz", "gks"):
        exprs = {}
        for m in re.finditer(name + r"\[(\d)\]\s*=\s*(.*?);", text, re.S):
            body = " ".join(re.sub(r"//.*", "", ln) for ln in m.group(2).splitlines())
            body = re.sub(r"([xy])\[(\d)\]", r"\1\2", body)
            exprs[int(m.group(1))] = compile(body, f"{name}[{m.group(1)}]", "eval")
        assert sorted(exprs) == list(range(9)), name
        out[name] = exprs
    return out


def reference_sums(poly, tx, y, zeta, sigma, area, mask, eps, collocated, tgt_idx):
    """(n x 12) sums in extended precision: u, v, w, then the gradient tensor."""
    epssq = LD(eps) * LD(eps)
    Y = [LD(1) * y[:, k][None, :] for k in range(3)]
    keep = (mask == 0)[None, :]
    out = np.zeros((tx.shape[0], 12), dtype=LD)
    for r0 in range(0, tx.shape[0], 64):
        X = [LD(1) * tx[r0:r0 + 64, k][:, None] for k in range(3)]
        w = keep & np.ones((len(X[0]), 1), bool)
        if collocated:
            rows = tgt_idx[r0:r0 + 64]
            w[np.arange(len(rows)), rows] = False
        dot = X[0] * Y[0] + X[1] * Y[1] + X[2] * Y[2]
        base = 1 - dot + epssq
        rot = -(LD(1) * zeta)[None, :] * area[None, :]
        pot = -(LD(1) * sigma)[None, :] * area[None, :]
        sz = rot / (4 * PI * base)
        ss = pot / (4 * PI * base)
        cross = [X[1] * Y[2] - X[2] * Y[1], X[2] * Y[0] - X[0] * Y[2], X[0] * Y[1] - X[1] * Y[0]]
        for j in range(3):
            proj = sum(((1 if k == j else 0) - X[j] * X[k]) * Y[k] for k in range(3))
            out[r0:r0 + 64, j] = np.sum(np.where(w, cross[j] * sz + proj * ss, 0), axis=1)
        env = {"epssq": epssq, "square": lambda a: a * a, "cube": lambda a: a * a * a}
        env.update({f"x{k}": X[k] for k in range(3)})
        env.update({f"y{k}": Y[k] for k in range(3)})
        den2 = 1 / (4 * PI * (base * base))
        for k in range(9):
            gkz = eval(poly["gkz"][k], {}, env) * den2
            gks = eval(poly["gks"][k], {}, env) * den2
            out[r0:r0 + 64, 3 + k] = np.sum(np.where(w, gkz * rot + gks * pot, 0), axis=1)
    return out


def main():
    header = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(
        "/root/reference/src/lpm_swe_kernels.hpp")
    poly = read_polynomials(header)
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, 3, 1.0)
    rng = np.random.default_rng(2026)
    # smooth vorticity and divergence plus noise, on every face slot
    zeta = 2 * fx[:, 2] + np.sin(3 * fx[:, 0]) + 0.1 * rng.standard_normal(fx.shape[0])
    sigma = 0.5 * fx[:, 0] * fx[:, 1] + np.cos(2 * fx[:, 2]) + 0.1 * rng.standard_normal(fx.shape[0])
    # leaf faces only: a divided (parent) slot coincides with its central
    # child, where the reference's kernels divide by zero
    ftgt = np.sort(rng.choice(np.flatnonzero(fm == 0), 256, replace=False))
    cases = {}
    for eps in (0.0, 0.05):
        v = reference_sums(poly, vx, fx, zeta, sigma, fa, fm, eps, False, None)
        f = reference_sums(poly, fx[ftgt], fx, zeta, sigma, fa, fm, eps,
                           abs(eps) < np.finfo(np.float64).eps, ftgt)
        tag = "e0" if eps == 0 else "e5"
        cases[f"vert_{tag}"] = v.astype(np.float64)
        cases[f"face_{tag}"] = f.astype(np.float64)
    np.savez_compressed(HERE / "swe_sphere_icos_l3.npz", vx=vx, fx=fx, fa=fa, fm=fm, zeta=zeta,
                        sigma=sigma, face_targets=ftgt, **cases)
    print("wrote", HERE / "swe_sphere_icos_l3.npz")


if __name__ == "__main__":
    main()

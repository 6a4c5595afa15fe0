"""Generates tests/golden/swe_sphere_icos_l3.npz: the reference's spherical SWE
pair formulas (src/lpm_swe_kernels.hpp: kzeta_sphere :63-76, ksigma_sphere
:87-108, grad_kzeta :114-150, grad_ksigma :179-325, summed as in
SphereSweDirectSumReducer :608-619) evaluated in extended precision on FP64
inputs.

    python tests/golden/make_swe_sphere_golden.py <lpm>/src/lpm_swe_kernels.hpp

The velocity-gradient entries are not restated: the script reads the
reference header as text, parses each `gkz[k] = ...;` / `gks[k] = ...;`
expression into a syntax tree, checks that it holds nothing but arithmetic
(+, -, *, /, unary signs, numbers, the names x0..x2, y0..y2, epssq and calls
of square/cube) and evaluates that tree itself with np.longdouble (64-bit
significand on x86-64) -- the text is never handed to eval -- so the fixture
holds the reference's own polynomials to ~1e-18 relative per pair.  The FP64
oracle and the CUDA path, which evaluate equivalent compact forms, are pinned
against these values.  The mesh is the reference's (the oracle's tree_init
restatement from the reference's seed file).
"""
import ast
import operator
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import lpm_oracle as O  # noqa: E402

_BINOPS = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul,
           ast.Div: operator.truediv}
_UNOPS = {ast.USub: operator.neg, ast.UAdd: operator.pos}
_FUNCS = {"square": lambda a: a * a, "cube": lambda a: a * a * a}
_NAMES = {"epssq"} | {f"{c}{k}" for c in "xy" for k in range(3)}


def check_tree(node):
    """Raises ValueError unless the expression is plain arithmetic."""
    if isinstance(node, ast.Expression):
        return check_tree(node.body)
    if isinstance(node, ast.BinOp) and type(node.op) in _BINOPS:
        check_tree(node.left)
        check_tree(node.right)
    elif isinstance(node, ast.UnaryOp) and type(node.op) in _UNOPS:
        check_tree(node.operand)
    elif isinstance(node, ast.Constant) and type(node.value) in (int, float):
        pass
    elif isinstance(node, ast.Name) and node.id in _NAMES:
        pass
    elif (isinstance(node, ast.Call) and isinstance(node.func, ast.Name)
          and node.func.id in _FUNCS and len(node.args) == 1 and not node.keywords):
        check_tree(node.args[0])
    else:
        raise ValueError(f"unexpected syntax in a gradient polynomial: {ast.dump(node)[:80]}")
    return node


def evaluate(node, env):
    """Evaluates a tree accepted by check_tree with the arrays in env."""
    if isinstance(node, ast.Expression):
        return evaluate(node.body, env)
    if isinstance(node, ast.BinOp):
        return _BINOPS[type(node.op)](evaluate(node.left, env), evaluate(node.right, env))
    if isinstance(node, ast.UnaryOp):
        return _UNOPS[type(node.op)](evaluate(node.operand, env))
    if isinstance(node, ast.Constant):
        return LD(node.value)
    if isinstance(node, ast.Name):
        return env[node.id]
    return _FUNCS[node.func.id](evaluate(node.args[0], env))

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
            exprs[int(m.group(1))] = check_tree(ast.parse(body.strip(), mode="eval"))
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
        env = {"epssq": epssq}
        env.update({f"x{k}": X[k] for k in range(3)})
        env.update({f"y{k}": Y[k] for k in range(3)})
        den2 = 1 / (4 * PI * (base * base))
        for k in range(9):
            gkz = evaluate(poly["gkz"][k], env) * den2
            gks = evaluate(poly["gks"][k], env) * den2
            out[r0:r0 + 64, 3 + k] = np.sum(np.where(w, gkz * rot + gks * pot, 0), axis=1)
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_swe_sphere_golden.py <the reference's src/lpm_swe_kernels.hpp>")
    poly = read_polynomials(Path(sys.argv[1]))
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 3, 1.0)
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

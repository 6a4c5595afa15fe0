"""CPU pins of the far-field oracle (oracle/farfield_oracle.py): the order-4
expansion converges to the exact cell sum like rho^5, the correction built
from the exact residual reproduces the exact velocity, and the features are
invariant under rotations about the cell normal (the canonical frame)."""
import math

import numpy as np


def _cap(rng, n, center, radius):
    """n points on the unit sphere within `radius` of `center`."""
    c = center / np.linalg.norm(center)
    a = np.array([0.0, 0.0, 1.0]) if abs(c[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    e1 = np.cross(a, c)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(c, e1)
    r = radius * np.sqrt(rng.uniform(0, 1, n))
    t = rng.uniform(0, 2 * math.pi, n)
    p = c + r[:, None] * (np.cos(t)[:, None] * e1 + np.sin(t)[:, None] * e2)
    return p / np.linalg.norm(p, axis=1)[:, None]


def _targets(cell, rho, n, rng):
    """Unit-sphere targets at distance h / rho from the cell centre."""
    c = cell["c"]
    D = cell["h"] / rho
    cn = np.linalg.norm(c)
    ca = (1 + cn * cn - D * D) / (2 * cn)
    sa = math.sqrt(1 - ca * ca)
    e1, e2, nn = cell["Q"]
    b = rng.uniform(0, 2 * math.pi, n)
    x = ca * nn + sa * (np.cos(b)[:, None] * e1 + np.sin(b)[:, None] * e2)
    return x / np.linalg.norm(x, axis=1)[:, None]


def test_expansion_converges():
    import farfield_oracle as fo

    rng = np.random.default_rng(0)
    y = _cap(rng, 200, np.array([0.3, -0.2, 0.9]), 0.08)
    g = rng.uniform(-1, 1, 200)
    cell = fo.cell_record(y, g)
    errs = []
    for rho in (0.4, 0.2, 0.1):
        x = _targets(cell, rho, 64, rng)
        ue = fo.exact(y, g, x, 2e-4)
        ua = fo.expansion(cell, x, 2e-4)
        errs.append(np.max(np.linalg.norm(ua - ue, axis=1)) / np.max(np.linalg.norm(ue, axis=1)))
    assert errs[0] < 2e-2 and errs[2] < 1e-4
    # fifth-order truncation: halving rho gains about 2^5
    assert errs[0] / errs[1] > 12 and errs[1] / errs[2] > 12


def test_correction_reproduces_exact():
    import farfield_oracle as fo

    rng = np.random.default_rng(1)
    y = _cap(rng, 64, np.array([-0.5, 0.5, 0.2]), 0.1)
    g = rng.uniform(0.5, 1.5, 64)
    cell = fo.cell_record(y, g)
    x = _targets(cell, 0.3, 32, rng)
    c0 = 2e-4
    t = fo.residual_target(cell, y, g, x, c0)
    u = fo.expansion(cell, x, c0) + fo.correction(cell, x, t, 1.0)
    ue = fo.exact(y, g, x, c0)
    assert np.max(np.abs(u - ue)) < 1e-12 * np.max(np.abs(ue)) + 1e-14


def test_features_invariant_under_rotation_about_the_normal():
    import farfield_oracle as fo

    rng = np.random.default_rng(2)
    y = _cap(rng, 64, np.array([0.1, 0.7, 0.6]), 0.1)
    g = rng.uniform(-1, 1, 64)
    cell = fo.cell_record(y, g)
    x = _targets(cell, 0.25, 8, rng)
    f0 = fo.features(cell, x, 0.01)
    t0 = fo.residual_target(cell, y, g, x, 2e-4)
    n = cell["Q"][2]
    al = 0.7
    K = np.array([[0, -n[2], n[1]], [n[2], 0, -n[0]], [-n[1], n[0], 0]])
    Rm = np.eye(3) + math.sin(al) * K + (1 - math.cos(al)) * K @ K
    cell2 = fo.cell_record(y @ Rm.T, g)
    f1 = fo.features(cell2, x @ Rm.T, 0.01)
    t1 = fo.residual_target(cell2, y @ Rm.T, g, x @ Rm.T, 2e-4)
    assert np.allclose(f0, f1, atol=1e-10)
    assert np.allclose(t0, t1, atol=1e-8 * np.max(np.abs(t0)))

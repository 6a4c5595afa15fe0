"""CPU pins of the network oracle (oracle/mlp_oracle.py): its backward pass
against central finite differences of its own loss (plain FP64), and its BF16
rounding against torch's."""
import numpy as np
import pytest


def test_oracle_gradient_finite_differences():
    import mlp_oracle as mo

    rng = np.random.default_rng(0)
    w = rng.uniform(-0.2, 0.2, 40960)
    x = rng.normal(0, 1, (6, 48))
    x[:, 40] = 1.0
    x[:, 41:] = 0.0
    y = rng.normal(0, 1, (6, 3))
    g = mo.grad(w, x, y, rounding=False)
    # a few entries of every matrix, including bias columns and the constant unit
    idx = [0, 40, 129 * 48 - 1, 6144 + 5, 6144 + 127, 6144 + 16384 + 200,
           6144 + 2 * 16384 + 3, 6144 + 2 * 16384 + 127, 6144 + 2 * 16384 + 2 * 128 + 64]
    for i in idx:
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (mo.loss(wp, x, y, False) - mo.loss(wm, x, y, False)) / (2 * h)
        assert g[i] == pytest.approx(fd, rel=1e-5, abs=1e-9), i
    # rows that produce the constant unit get no gradient; unused outputs neither
    assert np.all(g[127 * 48:128 * 48] == 0)
    assert np.all(g[6144 + 2 * 16384 + 3 * 128:] == 0)


def test_bf16_rounding_matches_torch():
    import torch

    import mlp_oracle as mo

    rng = np.random.default_rng(1)
    a = (rng.normal(0, 1, 10000) * 10.0 ** rng.integers(-8, 8, 10000)).astype(np.float32)
    ref = torch.tensor(a).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(mo.bf16(a), ref)

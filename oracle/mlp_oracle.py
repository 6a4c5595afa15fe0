"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the learned far-field
network's forward pass and gradient, with BF16 rounding at the same points as
the tensor-core kernels (lpm_gb300/csrc/mlp.cu), so the GPU gradient can be
checked against it.  Imported by tests only; never by the product path.

Network: 48 inputs -> 128 -> 128 -> 128 -> 16 (first 3 outputs used), SiLU.
Input 40 and hidden unit 127 of every layer are the constant 1 (the next
weight matrix's column that multiplies them is the bias).  Loss: mean over the
n rows of the summed squared error of the 3 outputs.
"""
from __future__ import annotations

import numpy as np

BIAS_HID = 127


def bf16(a) -> np.ndarray:
    """Round float32 values to BF16 (nearest, ties to even), as float64."""
    f = np.ascontiguousarray(np.asarray(a, np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def split(w):
    w = np.asarray(w, np.float64)
    a, b, c = 128 * 48, 128 * 48 + 128 * 128, 128 * 48 + 2 * 128 * 128
    return (w[:a].reshape(128, 48), w[a:b].reshape(128, 128), w[b:c].reshape(128, 128),
            w[c:].reshape(16, 128))


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(w, x, rounding=True):
    """Returns the outputs (n x 16) and the intermediates of the forward pass
    (rounding=False: plain FP64, for finite-difference checks of the oracle)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, W2, W3, W4 = (r(m) for m in split(w))
    X = r(x)
    Z1 = X @ W1.T
    A1 = r(silu(Z1))
    A1[:, BIAS_HID] = 1.0
    Z2 = A1 @ W2.T
    A2 = r(silu(Z2))
    A2[:, BIAS_HID] = 1.0
    Z3 = A2 @ W3.T
    A3 = r(silu(Z3))
    A3[:, BIAS_HID] = 1.0
    Y = A3 @ W4.T
    return Y, (X, Z1, A1, Z2, A2, Z3, A3, W1, W2, W3, W4)


def grad(w, x, y, rounding=True):
    """Gradient of mean_rows sum_k (out_k - y_k)^2 w.r.t. the master weights."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    n = x.shape[0]
    Y, (X, Z1, A1, Z2, A2, Z3, A3, W1, W2, W3, W4) = forward(w, x, rounding)
    dY = np.zeros_like(Y)
    dY[:, :3] = r(2.0 * (Y[:, :3] - np.asarray(y, np.float64)) / n)
    gW4 = dY.T @ A3
    dZ3 = r(dY @ W4 * silu_grad(Z3))
    dZ3[:, BIAS_HID] = 0.0
    gW3 = dZ3.T @ A2
    dZ2 = r(dZ3 @ W3 * silu_grad(Z2))
    dZ2[:, BIAS_HID] = 0.0
    gW2 = dZ2.T @ A1
    dZ1 = r(dZ2 @ W2 * silu_grad(Z1))
    dZ1[:, BIAS_HID] = 0.0
    gW1 = dZ1.T @ X
    return np.concatenate([gW1.ravel(), gW2.ravel(), gW3.ravel(), gW4.ravel()])


def loss(w, x, y, rounding=True):
    Y, _ = forward(w, x, rounding)
    return float(np.mean(np.sum((Y[:, :3] - y) ** 2, axis=1)))

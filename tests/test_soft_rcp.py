"""The FMA-pipe reciprocal of the planar velocity + stream-function kernel
(neg_rcp2 in lpm_gb300/csrc/nbody.cuh), restated in numpy with the header's
own seed constant: the bit-level seed is within 5.1 % of -1/q, and three
Newton steps y <- y + y (1 + q y) bring it within 0.5 ulp (6e-8 relative)
of 1/q in FP64, over the range of q the chord sums pass (c0 = eps^2 plus a
1e-30 floor, up to the squared diameter of a domain far larger than the
tests')."""
import re
from pathlib import Path

import numpy as np

SRC = Path(__file__).resolve().parents[1] / "lpm_gb300" / "csrc" / "nbody.cuh"


def seed_constant():
    body = SRC.read_text().split("u64 neg_rcp2(", 1)[1].split("\n}", 1)[0]
    consts = set(re.findall(r"0x([0-9A-Fa-f]{8})u", body))
    assert len(consts) == 1, consts
    assert "for (int it = 0; it < 3; ++it) y = fma2(y, fma2(q, y, one2), y);" in body
    return np.uint32(int(consts.pop(), 16))


def fma32(a, b, c):
    # a*b + c rounded once to FP32 (the FP64 product of two floats is exact)
    return (a.astype(np.float64) * b + c).astype(np.float32)


def neg_rcp(q):
    y = (seed_constant() - q.view(np.uint32)).view(np.float32)
    seed = y.copy()
    for _ in range(3):
        y = fma32(y, fma32(q, y, np.float32(1.0)), y)
    return seed, y


def test_seed_and_newton_steps():
    rng = np.random.default_rng(3)
    q = np.concatenate([np.exp(rng.uniform(np.log(1e-30), np.log(1e6), 1_000_000)).astype(np.float32),
                        np.float32(2.0) ** np.arange(-99, 19, dtype=np.float32),
                        np.nextafter(np.float32(2.0) ** np.arange(-99, 19, dtype=np.float32),
                                     np.float32(0))])
    seed, y = neg_rcp(q)
    q64 = q.astype(np.float64)
    assert np.abs(-seed.astype(np.float64) * q64 - 1).max() < 0.051
    exact = 1.0 / q64
    r = -y.astype(np.float64)
    assert np.abs(r * q64 - 1).max() < 6e-8
    ulp = np.spacing(exact.astype(np.float32)).astype(np.float64)
    assert (np.abs(r - exact) <= 0.5 * ulp + 1e-300).mean() > 0.999
    assert (np.abs(r - exact) <= ulp).all()


def test_bench_bound_matches_the_kernel_pattern():
    """bench.py's XU bound for the planar step counts the MUFU reciprocals the
    final kernel keeps: the popcount of soft_rcp_sources' pattern (of 8)."""
    body = SRC.read_text().split("constexpr unsigned soft_rcp_sources(", 1)[1].split("\n}", 1)[0]
    pattern = int(re.search(r"\? 0x([0-9A-Fa-f]+)u : 0u", body).group(1), 16)
    bench = (Path(__file__).resolve().parents[1] / "bench.py").read_text()
    m = re.search(r"mufu_final = 2 - (\d) / 8", bench)
    assert m and int(m.group(1)) == bin(pattern).count("1")

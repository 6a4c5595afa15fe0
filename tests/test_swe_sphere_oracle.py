"""CPU pins of the spherical SWE oracle (oracle_swe_sphere_sums).

1. Against the reference's own pair polynomials (grad_kzeta / grad_ksigma,
   src/lpm_swe_kernels.hpp:114-325, with kzeta_sphere / ksigma_sphere
   :63-108) evaluated in extended precision by tests/golden/
   make_swe_sphere_golden.py on an icosahedral level-3 mesh: vertex sums and
   face sums (the collocated i == j skip at eps = 0), eps = 0 and 0.05.
2. With zero divergence the velocity equals the incompressible-2D sphere sums
   (Incompressible2DKernels<SphereGeometry>, the same kernel).
3. Tangency: u . x = 0 at every target.

Finding (test_gradient_signs): the summed tensor M = sum gkz rot + gks pot
with rot = -zeta A, pot = -sigma A equals -(grad u_zeta) P + (grad u_sigma) P,
where u_zeta, u_sigma are the rotational and divergent parts of the velocity
the same functor returns and P = I - x x^T: grad_kzeta carries the opposite
sign of the rotational velocity's surface gradient.  The double dot product
sum_ij M_ij M_ji therefore differs from that of the velocity's gradient by
4 tr(A B) when both parts are present.  Oracle and GPU path reproduce the
reference's tensor.
"""
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "swe_sphere_icos_l3.npz"


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("eps,tag", [(0.0, "e0"), (0.05, "e5")])
def test_oracle_matches_reference_polynomials(oracle, eps, tag):
    g = np.load(GOLD)
    v = oracle.swe_sphere_sums(g["vx"], g["fx"], g["zeta"], g["sigma"], g["fa"], g["fm"], eps)
    ft = g["face_targets"]
    f = oracle.swe_sphere_sums(g["fx"], g["fx"], g["zeta"], g["sigma"], g["fa"], g["fm"], eps,
                               collocated=eps == 0)[ft]
    for got, ref in ((v, g[f"vert_{tag}"]), (f, g[f"face_{tag}"])):
        assert _rel(got[:, :3], ref[:, :3]) < 1e-13
        assert _rel(got[:, 3:], ref[:, 3:]) < 1e-12
        assert _rel(oracle.double_dot(got[:, 3:]), oracle.double_dot(ref[:, 3:])) < 1e-12


def _icos(level):
    import lpm_oracle as O

    return O.mesh(O.MESH_ICOS_TRI, level, 1.0)


def test_rotational_velocity_matches_ic2d_and_is_tangent(oracle):
    vx, fx, fa, fm = _icos(3)
    zeta = np.sin(2 * fx[:, 0]) + fx[:, 2]
    out = oracle.swe_sphere_sums(vx, fx, zeta, np.zeros_like(zeta), fa, fm, 0.03)
    u, _ = oracle.ic2d_passive_sums(vx, fx, zeta, fa, fm, 0.03)
    assert _rel(out[:, :3], u) < 1e-13
    sigma = np.cos(3 * fx[:, 1])
    out = oracle.swe_sphere_sums(vx, fx, zeta, sigma, fa, fm, 0.03)
    tang = np.abs(np.sum(out[:, :3] * vx, 1)).max() / np.abs(out[:, :3]).max()
    assert tang < 1e-13


def test_gradient_signs(oracle):
    """M = -(grad u_zeta) P for a rotational field, +(grad u_sigma) P for a
    divergent one (central differences of the oracle's own velocity)."""
    vx, fx, fa, fm = _icos(3)
    eps = 0.1
    zeta = np.sin(2 * fx[:, 0]) + fx[:, 2]
    sigma = np.cos(3 * fx[:, 1]) * fx[:, 0]
    zero = np.zeros_like(zeta)
    x = vx[::37]
    P = np.eye(3)[None] - x[:, :, None] * x[:, None, :]
    h = 1e-5
    for z, s, sign in ((zeta, zero, -1.0), (zero, sigma, 1.0)):
        M = oracle.swe_sphere_sums(x, fx, z, s, fa, fm, eps)[:, 3:].reshape(-1, 3, 3)
        J = np.zeros_like(M)
        for ax in range(3):
            e = np.zeros(3)
            e[ax] = h
            up = oracle.swe_sphere_sums(x + e, fx, z, s, fa, fm, eps)[:, :3]
            dn = oracle.swe_sphere_sums(x - e, fx, z, s, fa, fm, eps)[:, :3]
            J[:, :, ax] = (up - dn) / (2 * h)
        want = sign * J @ P
        assert _rel(M, want) < 1e-6
        assert _rel(M, -want) > 0.5

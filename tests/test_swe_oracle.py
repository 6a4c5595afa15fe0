"""CPU pins of the planar SWE oracle (oracle_swe_plane_sums): with zero
divergence its velocity and stream function equal the incompressible-2D plane
sums (pinned elsewhere); its divergent part is the rotated potential field;
and the PSE sum of s = x^2 + y^2 is the Laplacian 4 times pse_eps^2.

Finding: planar_swe_sums_rhs_pse (src/lpm_swe_kernels.hpp:469-471) divides
the PSE sum by pse_eps^2 once; the two-dimensional kernel's own 1/pse_eps^2
scaling is absent, so its "laplacian" is pse_eps^2 times the Laplacian.  The
oracle and the GPU path reproduce the reference's value."""
import math

import numpy as np


def _mesh(level):
    import lpm_oracle as O

    vx, fx, fa, fm = O.mesh(O.MESH_QUAD_RECT, level, 4.0)
    return vx, fx, fa, fm


def test_swe_rotational_part_matches_ic2d(oracle):
    vx, fx, fa, fm = _mesh(4)
    rng = np.random.default_rng(0)
    zeta = np.exp(-np.sum(fx ** 2, 1))
    sigma = np.zeros(fx.shape[0])
    s = rng.normal(size=fx.shape[0])
    out = oracle.swe_plane_sums(vx, np.zeros(vx.shape[0]), fx, zeta, sigma, fa, fm, s, 0.05, 0.3)
    u, psi = oracle.ic2d_passive_sums(vx, fx, zeta, fa, fm, 0.05)
    assert np.allclose(out[:, 0:2], u, rtol=1e-12, atol=1e-14)
    assert np.allclose(out[:, 7], psi, rtol=1e-12, atol=1e-14)
    assert np.all(out[:, 8] == 0)


def test_swe_divergent_part_is_potential_flow(oracle):
    """With zeta = 0 the velocity is the gradient of the potential phi
    (u = -grad of -log/4pi ...): it equals the rotational field of the same
    strength turned by 90 degrees."""
    vx, fx, fa, fm = _mesh(3)
    sig = np.cos(fx[:, 0]) * np.exp(-np.sum(fx ** 2, 1) / 4)
    a = oracle.swe_plane_sums(vx, np.zeros(vx.shape[0]), fx, np.zeros_like(sig), sig, fa, fm,
                              np.zeros_like(sig), 0.1, 0.3)
    b = oracle.swe_plane_sums(vx, np.zeros(vx.shape[0]), fx, sig, np.zeros_like(sig), fa, fm,
                              np.zeros_like(sig), 0.1, 0.3)
    # (u, v)_sigma = (v, -u)_zeta ; dudx_sigma = dv/dx_zeta etc.
    assert np.allclose(a[:, 0], b[:, 1], rtol=1e-12, atol=1e-14)
    assert np.allclose(a[:, 1], -b[:, 0], rtol=1e-12, atol=1e-14)
    assert np.allclose(a[:, 8], b[:, 7], rtol=1e-12, atol=1e-14)


def test_pse_laplacian_of_quadratic(oracle):
    vx, fx, fa, fm = _mesh(6)
    s = np.sum(fx ** 2, 1)
    h = math.sqrt(fa[fm == 0].mean())
    pse_eps = 2.0 * h
    inner = np.nonzero(np.max(np.abs(vx), 1) < 2.0)[0]
    out = oracle.swe_plane_sums(vx[inner], np.sum(vx[inner] ** 2, 1), fx, np.zeros_like(s),
                                np.zeros_like(s), fa, fm, s, 0.0, pse_eps)
    # eighth-order PSE: exact for a quadratic up to quadrature error
    assert np.allclose(out[:, 6] / pse_eps ** 2, 4.0, rtol=1e-6)

"""Pins of the FP64 CPU oracle against the reference's own known answers.

The reference holds no golden vectors for this path; these checks come from
its examples and tests:
  - solid-body rotation: u = Omega (-y, x, 0) and psi = 2 pi z
    (examples/bve_rotation.cpp:147-166), converging with the mesh;
  - Rossby-Haurwitz 5-4 analytic velocity (src/lpm_velocity_gallery.hpp:270-287);
  - tangency u.x = 0 (src/lpm_sphere_functions.hpp:59-78);
  - second-order time convergence of Incompressible2DRK2 on the cubed sphere,
    depth 4, eps 0, t_f 0.5, steps {15, 30, 60} (tests/lpm_ic2d_tests.cpp:165-188);
  - BVE RK4 is fourth order in time;
  - ErrNorms definitions (src/lpm_error.hpp:81-91).
"""
import math

import numpy as np
import pytest

import lpm_oracle as O

OMEGA = 2 * math.pi


def solid_body(level):
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, level, 1.0)
    zf = O.ic_eval(O.IC_SOLID_BODY, (), fx)
    return vx, fx, fa, fm, zf


def test_solid_body_rotation_velocity_and_stream_fn(oracle):
    errs_u, errs_psi = [], []
    for level in (2, 3, 4):
        vx, fx, fa, fm, zf = solid_body(level)
        psi, u = oracle.bve_vertex_solve(vx, fx, zf, fa, fm)
        exact = np.stack([-OMEGA * vx[:, 1], OMEGA * vx[:, 0], 0 * vx[:, 0]], 1)
        errs_u.append(oracle.err_norms(u, exact)[2])
        errs_psi.append(oracle.err_norms(psi, 2 * math.pi * vx[:, 2])[2])
    assert errs_u[-1] < 5e-3 and errs_u[0] > errs_u[1] > errs_u[2]
    # the stream function converges at second order (error / 4 per level)
    assert errs_psi[-1] < 1e-3
    rates = [math.log2(errs_psi[i] / errs_psi[i + 1]) for i in range(2)]
    assert min(rates) > 1.9


def test_rossby_haurwitz_velocity(oracle):
    w = OMEGA / 12.5
    errs = []
    for level in (3, 4):
        vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, level, 1.0)
        zf = O.ic_eval(O.IC_RH54, (w, -w), fx)
        _, u = oracle.bve_vertex_solve(vx, fx, zf, fa, fm, want_psi=False)
        lat, lon = np.arcsin(vx[:, 2]), np.arctan2(vx[:, 1], vx[:, 0])
        amp, u0 = -w, w
        uu = amp * 0.5 * np.cos(4 * lon) * np.cos(lat) ** 3 * (5 * np.cos(2 * lat) - 3)
        vv = amp * 4 * np.cos(lat) ** 3 * np.sin(lat) * np.sin(4 * lon)
        exact = np.stack([-u0 * vx[:, 1] - uu * np.sin(lon) - vv * np.sin(lat) * np.cos(lon),
                          u0 * vx[:, 0] + uu * np.cos(lon) - vv * np.sin(lat) * np.sin(lon),
                          vv * np.cos(lat)], 1)
        errs.append(oracle.err_norms(u, exact)[1])
    assert errs[1] < 3e-3 and errs[1] < 0.6 * errs[0]


def test_tangency(oracle):
    vx, fx, fa, fm, zf = solid_body(3)
    zf = zf + np.random.default_rng(1).standard_normal(zf.shape)
    _, u = oracle.bve_vertex_solve(vx, fx, zf, fa, fm, want_psi=False)
    assert np.abs((u * vx).sum(1)).max() < 1e-12 * np.abs(u).max() * 100


def test_masked_and_self_rules(oracle):
    """Masked slots never contribute; collocated BVE skips i == j; the ic2d
    active sums keep the self term for eps > 0 (psi gets -log(eps^2)/4pi Gamma_i)."""
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    zf = np.random.default_rng(2).standard_normal(fx.shape[0])
    psi_a, u_a = oracle.bve_face_solve(fx, zf, fa, fm)
    zf2 = zf.copy()
    zf2[fm == 1] = 1e6  # masked values must not matter
    psi_b, u_b = oracle.bve_face_solve(fx, zf2, fa, fm)
    leaf = fm == 0
    assert np.array_equal(u_a[leaf], u_b[leaf]) and np.array_equal(psi_a[leaf], psi_b[leaf])
    eps = 0.05
    _, p_incl = oracle.ic2d_active_sums(fx, zf, fa, fm, eps, self_rule=0)
    _, p_skip = oracle.ic2d_active_sums(fx, zf, fa, fm, eps, self_rule=1)
    gam = zf * fa
    arg = 1 - (fx * fx).sum(1) + eps * eps
    self_term = (-np.log(arg) / (4 * math.pi)) * gam
    assert np.allclose((p_incl - p_skip)[leaf], self_term[leaf], rtol=1e-10, atol=1e-14)


def test_ic2d_rk2_time_convergence(oracle):
    """tests/lpm_ic2d_tests.cpp:165-188 on the oracle: rate > 1.95."""
    vx, fx, fa, fm = O.mesh(O.MESH_CUBED_SPHERE, 4, 1.0)
    params = (4 * math.pi, 4.0, 0.0, math.pi / 20, 0.0, 0.0)  # GaussianVortexSphere()
    vz, fz = O.ic_eval(O.IC_GAUSSIAN_SPHERE, params, vx), O.ic_eval(
        O.IC_GAUSSIAN_SPHERE, params, fx)
    tf, nsteps = 0.5, (15, 30, 60)

    def run(n):
        s = oracle.IC2DState(vx, vz, fx, fz, fa, fm, 0.0, OMEGA)
        s.init_direct_sums()
        for _ in range(n):
            s.step(tf / n)
        return s.fx

    ref = run(nsteps[-1])
    leaf = fm == 0
    errs = []
    for n in nsteps[:-1]:
        errs.append(oracle.err_norms(run(n)[leaf], ref[leaf], fa[leaf]))
    dts = [tf / n for n in nsteps[:-1]]
    for k in range(3):  # l1, l2, linf
        rate = math.log(errs[0][k] / errs[1][k]) / math.log(dts[0] / dts[1])
        assert rate > 1.95, (k, rate)


def test_bve_rk4_fourth_order(oracle):
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    w = OMEGA / 12.5
    vz = O.ic_eval(O.IC_RH54, (w, -w), vx)
    fz = O.ic_eval(O.IC_RH54, (w, -w), fx)
    _, vu = oracle.bve_vertex_solve(vx, fx, fz, fa, fm, want_psi=False)
    _, fu = oracle.bve_face_solve(fx, fz, fa, fm, want_psi=False)
    leaf = fm == 0
    tf = 0.4

    def run(n):
        s = oracle.BVEState(vx, vz, vu, fx, fz, fu, fa, fm)
        for _ in range(n):
            s.step(tf / n, OMEGA, fix_facevort3=True)
        return s.fx[leaf]

    ref, a, b = run(32), run(4), run(8)
    ea, eb = np.abs(a - ref).max(), np.abs(b - ref).max()
    assert math.log2(ea / eb) > 3.5


def test_facevort3_quirk_changes_only_faces(oracle):
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 2, 1.0)
    fz = np.random.default_rng(4).standard_normal(fx.shape[0])
    vz = np.zeros(vx.shape[0])
    _, vu = oracle.bve_vertex_solve(vx, fx, fz, fa, fm, want_psi=False)
    _, fu = oracle.bve_face_solve(fx, fz, fa, fm, want_psi=False)
    a = oracle.BVEState(vx, vz, vu, fx, fz, fu, fa, fm)
    b = oracle.BVEState(vx, vz, vu, fx, fz, fu, fa, fm)
    a.step(0.01, OMEGA, fix_facevort3=False)
    b.step(0.01, OMEGA, fix_facevort3=True)
    leaf = fm == 0
    assert np.array_equal(a.vx, b.vx) and np.array_equal(a.fx[leaf], b.fx[leaf])
    assert not np.array_equal(a.fzeta[leaf], b.fzeta[leaf])


def test_err_norms_definition(oracle):
    rng = np.random.default_rng(5)
    exact = rng.standard_normal((50, 3))
    appx = exact + 1e-3 * rng.standard_normal((50, 3))
    w = rng.random(50)
    l1, l2, li = oracle.err_norms(appx, exact, w)
    em = np.linalg.norm(appx - exact, axis=1)
    xm = np.linalg.norm(exact, axis=1)
    assert math.isclose(l1, (em * w).sum() / (xm * w).sum(), rel_tol=1e-12)
    assert math.isclose(l2, math.sqrt((em ** 2 * w).sum() / (xm ** 2 * w).sum()), rel_tol=1e-12)
    assert math.isclose(li, em.max() / xm.max(), rel_tol=1e-12)


def test_invariants_definition(oracle):
    vx, fx, fa, fm = O.mesh(O.MESH_QUAD_RECT, 2, 4.0)
    rng = np.random.default_rng(6)
    z, u = rng.standard_normal(fx.shape[0]), rng.standard_normal((fx.shape[0], 2))
    tv, te, tk = oracle.invariants(z, u, fa, fm)
    leaf = fm == 0
    assert math.isclose(tv, (z * fa)[leaf].sum(), rel_tol=1e-12)
    assert math.isclose(te, 0.5 * (z * z * fa)[leaf].sum(), rel_tol=1e-12)
    assert math.isclose(tk, 0.5 * ((u * u).sum(1) * fa)[leaf].sum(), rel_tol=1e-12)


@pytest.mark.parametrize("targets", [1, 7, 100])
def test_target_subsets_match_full(oracle, targets):
    """Evaluating a target subset (the CPU-baseline sampling) gives the same
    rows as the full evaluation, bit for bit."""
    vx, fx, fa, fm, zf = solid_body(2)
    idx = np.random.default_rng(targets).choice(vx.shape[0], targets, replace=False)
    psi, u = oracle.bve_vertex_solve(vx, fx, zf, fa, fm)
    psi_s, u_s = oracle.bve_vertex_solve(vx, fx, zf, fa, fm, tgt_idx=idx)
    assert np.array_equal(u_s, u[idx]) and np.array_equal(psi_s, psi[idx])

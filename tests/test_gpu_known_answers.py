"""The CUDA path against the reference's own known answers, without the
oracle in between, on meshes finer than the oracle's pins can afford:
  - solid-body rotation zeta = 2 Omega z: u = Omega (-y, x, 0) and
    psi = 2 pi z (examples/bve_rotation.cpp:147-166), u converging and psi
    converging at second order with the mesh;
  - the Rossby-Haurwitz 5-4 analytic velocity (src/lpm_velocity_gallery.hpp:
    270-287), error falling with the mesh;
  - tangency u.x = 0 (src/lpm_sphere_functions.hpp:59-78).
Meshes and initial conditions come from the oracle's restatement of the
reference's seeds and vorticity gallery; errors are ErrNorms
(src/lpm_error.hpp:81-91) evaluated on the host.
"""
import math

import numpy as np
import pytest
import torch

import lpm_oracle as O
from lpm_gb300 import core
from lpm_gb300 import functors as F

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def vertex_solve(ctx, level, kind, params):
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, level, 1.0)
    zf = O.ic_eval(kind, params, fx)
    psi = torch.zeros(vx.shape[0], dtype=torch.float64, device="cuda")
    u = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
    F.bve_vertex_solve(ctx, psi, u, dev(vx), dev(fx), dev(zf), dev(fa), dev(fm))
    ctx.synchronize()
    return vx, psi.cpu().numpy(), u.cpu().numpy()


def linf(appx, exact):
    return O.err_norms(appx, exact)[2]


@pytest.mark.parametrize("precision", [core.FP64, core.FP32C])
def test_solid_body_rotation(gpu_ctx, precision):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    eu, ep = [], []
    for level in (4, 5, 6):
        vx, psi, u = vertex_solve(ctx, level, O.IC_SOLID_BODY, ())
        exact = np.stack([-OMEGA * vx[:, 1], OMEGA * vx[:, 0], 0 * vx[:, 0]], 1)
        eu.append(linf(u, exact))
        ep.append(linf(psi, 2 * math.pi * vx[:, 2]))
    assert eu[0] > eu[1] > eu[2] and eu[2] < 1.2e-3, eu  # level 6: 8.4e-4
    rates = [math.log2(ep[i] / ep[i + 1]) for i in range(2)]
    assert ep[2] < 4e-5 and min(rates) > 1.9, (ep, rates)  # level 6: 2.6e-5


@pytest.mark.parametrize("precision", [core.FP64, core.FP32C])
def test_rossby_haurwitz_analytic_velocity(gpu_ctx, precision):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    w = OMEGA / 12.5
    errs = []
    for level in (4, 5, 6):
        vx, _, u = vertex_solve(ctx, level, O.IC_RH54, (w, -w))
        lat, lon = np.arcsin(vx[:, 2]), np.arctan2(vx[:, 1], vx[:, 0])
        amp, u0 = -w, w
        uu = amp * 0.5 * np.cos(4 * lon) * np.cos(lat) ** 3 * (5 * np.cos(2 * lat) - 3)
        vv = amp * 4 * np.cos(lat) ** 3 * np.sin(lat) * np.sin(4 * lon)
        exact = np.stack([-u0 * vx[:, 1] - uu * np.sin(lon) - vv * np.sin(lat) * np.cos(lon),
                          u0 * vx[:, 0] + uu * np.cos(lon) - vv * np.sin(lat) * np.sin(lon),
                          vv * np.cos(lat)], 1)
        errs.append(O.err_norms(u, exact)[1])
    assert errs[0] > errs[1] > errs[2] and errs[2] < 5e-4, errs  # level 6: 3.3e-4


@pytest.mark.parametrize("precision,tol", [(core.FP64, 1e-13), (core.FP32C, 1e-13)])
def test_tangency(gpu_ctx, precision, tol):
    ctx = gpu_ctx
    ctx.set_precision(precision)
    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, 5, 1.0)
    zf = O.ic_eval(O.IC_SOLID_BODY, (), fx) + np.random.default_rng(1).standard_normal(fx.shape[0])
    u = torch.zeros(vx.shape[0], 3, dtype=torch.float64, device="cuda")
    F.bve_vertex_velocity(ctx, u, dev(vx), dev(fx), dev(zf), dev(fa), dev(fm))
    ctx.synchronize()
    un = u.cpu().numpy()
    assert np.abs((un * vx).sum(1)).max() < tol * np.abs(un).max()

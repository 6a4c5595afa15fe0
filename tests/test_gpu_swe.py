"""Planar SWE direct sums on the GPU against the FP64 oracle: vertex sums and
face sums (collocated i == j skip for eps = 0), every output, masked parent
slots excluded, FP64 parity 1e-12 (ErrNorms linf normalisation per output)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ["u", "du1dx1", "du1dx2", "du2dx1", "du2dx2", "laps", "psi", "phi"]


def _fields(level):
    from lpm_gb300 import core

    vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, level, 4.0)
    zeta = 2 * np.exp(-np.sum((fx - [1.0, 0.0]) ** 2, 1)) - 2 * np.exp(-np.sum((fx + [1.0, 0.0]) ** 2, 1))
    sigma = 0.3 * np.cos(fx[:, 0]) * np.exp(-np.sum(fx ** 2, 1) / 8)
    fs = 1 + 0.1 * np.exp(-np.sum(fx ** 2, 1))
    vs = 1 + 0.1 * np.exp(-np.sum(vx ** 2, 1))
    return vx, fx, fa, fm, zeta, sigma, fs, vs


def _check(got, ref9):
    cols = {"u": ref9[:, 0:2], "du1dx1": ref9[:, 2], "du1dx2": ref9[:, 3], "du2dx1": ref9[:, 4],
            "du2dx2": ref9[:, 5], "laps": ref9[:, 6], "psi": ref9[:, 7], "phi": ref9[:, 8]}
    for k in KEYS:
        g = got[k].cpu().numpy()
        r = cols[k]
        err = np.max(np.abs(g - r)) / max(np.max(np.abs(r)), 1e-300)
        assert err < 1e-12, (k, err)
    dd = ref9[:, 2] ** 2 + 2 * ref9[:, 3] * ref9[:, 4] + ref9[:, 5] ** 2
    g = got["ddot"].cpu().numpy()
    assert np.max(np.abs(g - dd)) / np.max(np.abs(dd)) < 1e-12


@pytest.mark.parametrize("eps", [0.0, 0.05])
def test_swe_plane_parity(gpu_ctx, oracle, eps):
    import torch

    from lpm_gb300 import functors as F

    vx, fx, fa, fm, zeta, sigma, fs, vs = _fields(5)
    h = math.sqrt(fa[fm == 0].mean())
    pse_eps = h ** 0.55  # PSEKernel::get_epsilon(dx, 11/20)
    d = torch.device("cuda", gpu_ctx.device)
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, sg=sigma, fs=fs, vs=vs).items()}
    gv = F.swe_plane_vertex_sums(gpu_ctx, T["vx"], T["vs"], T["fx"], T["z"], T["sg"], T["fa"],
                                 T["fm"], T["fs"], eps, pse_eps)
    gf = F.swe_plane_face_sums(gpu_ctx, T["fx"], T["z"], T["sg"], T["fa"], T["fm"], T["fs"], eps,
                               pse_eps)
    torch.cuda.synchronize()
    rv = oracle.swe_plane_sums(vx, vs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps, collocated=False)
    rf = oracle.swe_plane_sums(fx, fs, fx, zeta, sigma, fa, fm, fs, eps, pse_eps,
                               collocated=not eps > 0)
    _check(gv, rv)
    _check(gf, rf)


def test_swe_do_velocity_false_keeps_u(gpu_ctx):
    import torch

    from lpm_gb300 import core
    from lpm_gb300.core import check, lib, ptr, view

    vx, fx, fa, fm, zeta, sigma, fs, vs = _fields(3)
    d = torch.device("cuda", gpu_ctx.device)
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(fx=fx, fa=fa, fm=fm, z=zeta, sg=sigma, fs=fs).items()}
    u = torch.full((fx.shape[0], 2), 7.0, dtype=torch.float64, device=d)
    outs = [torch.zeros(fx.shape[0], dtype=torch.float64, device=d) for _ in range(8)]
    check(lib().lpm_swe_plane_face_sums(gpu_ctx.handle, view(u), *(ptr(o) for o in outs),
                                        view(T["fx"]), ptr(T["z"]), ptr(T["sg"]), ptr(T["fa"]),
                                        ptr(T["fm"]), ptr(T["fs"]), fx.shape[0], 0.05, 0.3, 0))
    torch.cuda.synchronize()
    assert bool((u == 7.0).all())
    with pytest.raises(core.LpmError):
        check(lib().lpm_swe_plane_face_sums(gpu_ctx.handle, view(u), *(ptr(o) for o in outs),
                                            view(T["fx"]), ptr(T["z"]), ptr(T["sg"]), ptr(T["fa"]),
                                            ptr(T["fm"]), ptr(T["fs"]), fx.shape[0], 0.05, 0.0, 1))

"""TEST INFRASTRUCTURE ONLY: numpy binding of the FP64 CPU oracle
(oracle/lpm_oracle.cpp).  Imported by the tests, the smoke check and the
CPU-baseline leg of bench.py as the checker; never by the product path.

Parity status: partially pinned (see the header of lpm_oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liblpm_oracle.so"
LIB_NATIVE = HERE / "build" / "liblpm_oracle_native.so"

_lib = None
_lib_native = None
_use_native = False


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def use_native(on: bool) -> None:
    """Route the calls below to the build tuned for this CPU (timing only)."""
    global _use_native
    _use_native = bool(on)


def lib() -> C.CDLL:
    global _lib, _lib_native
    if _use_native:
        if _lib_native is None:
            _lib_native = _load(LIB_NATIVE)
        return _lib_native
    if _lib is None:
        _lib = _load(LIB)
    return _lib


def _load(path: Path) -> C.CDLL:
    srcs = [HERE / "lpm_oracle.cpp", HERE / "lpm_oracle_mesh.cpp", HERE / "Makefile"]
    if not path.exists() or path.stat().st_mtime < max(p.stat().st_mtime for p in srcs):
        build()
    L = C.CDLL(str(path))
    vp, l, i, d = C.c_void_p, C.c_long, C.c_int, C.c_double
    sig = {
        "oracle_set_threads": [i],
        "oracle_swe_plane_sums": [l, vp, vp, l, vp, vp, vp, vp, vp, vp, d, d, i, vp],
        "oracle_swe_sphere_sums": [l, vp, l, vp, vp, vp, vp, vp, d, i, vp],
        "oracle_set_sphere_form": [i],
        "oracle_max_threads": [],
        "oracle_bve_vertex_solve": [vp, vp, vp, l, vp, vp, vp, vp, vp, l, i],
        "oracle_bve_face_solve": [vp, vp, l, vp, vp, vp, vp, vp, l, i],
        "oracle_ic2d_passive_sums": [i, vp, vp, vp, l, vp, vp, vp, vp, vp, d, l, i],
        "oracle_ic2d_active_sums": [i, vp, vp, l, vp, vp, vp, vp, vp, d, l, i, i],
        "oracle_bve_rk4_step": [l, vp, vp, vp, l, vp, vp, vp, vp, vp, d, d, d, i, i],
        "oracle_ic2d_init_direct_sums": [i, l, vp, vp, vp, l, vp, vp, vp, vp, vp, vp, d, i],
        "oracle_ic2d_rk2_step": [i, l, vp, vp, vp, vp, l, vp, vp, vp, vp, vp, vp, d, d, d, i],
        "oracle_invariants": [i, l, vp, vp, vp, vp, vp],
        "oracle_err_norms": [i, l, vp, vp, vp, vp, vp],
        "oracle_mesh_build": [i, i, i, l, l, l, vp, vp, vp, vp, d, i, l, l, vp, vp, vp, vp,
                              vp],
        "oracle_ic_eval": [i, vp, i, i, l, vp, vp],
    }
    ret_int = ("oracle_max_threads", "oracle_mesh_build", "oracle_ic_eval")
    for k, a in sig.items():
        f = getattr(L, k)
        f.argtypes = a
        f.restype = C.c_int if k in ret_int else None
    return L


def _p(a):
    return None if a is None else a.ctypes.data


def _f(a, shape=None):
    a = np.ascontiguousarray(a, np.float64)
    return a if shape is None else a.reshape(shape)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def set_sphere_form(chord: bool) -> None:
    """False: the reference's 1 - x.y (default); True: the chord form."""
    lib().oracle_set_sphere_form(int(bool(chord)))


class chord_form:
    """Context manager evaluating sphere kernels in the chord form."""

    def __enter__(self):
        set_sphere_form(True)
        return self

    def __exit__(self, *exc):
        set_sphere_form(False)
        return False


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def bve_vertex_solve(vx, fx, zeta, area, mask, want_u=True, want_psi=True, tgt_idx=None,
                     compensated=False):
    """BVEVertexSolve: returns (psi, u) over targets (tgt_idx subset if given)."""
    vx, fx, zeta, area = _f(vx), _f(fx), _f(zeta), _f(area)
    mask = np.ascontiguousarray(mask, np.uint8)
    idx = None if tgt_idx is None else np.ascontiguousarray(tgt_idx, np.int64)
    n = vx.shape[0] if idx is None else idx.shape[0]
    psi = np.zeros(n) if want_psi else None
    u = np.zeros((n, 3)) if want_u else None
    lib().oracle_bve_vertex_solve(_p(psi), _p(u), _p(vx), n, _p(idx), _p(fx), _p(zeta), _p(area),
                                  _p(mask), fx.shape[0], int(compensated))
    return psi, u


def bve_face_solve(fx, zeta, area, mask, want_u=True, want_psi=True, tgt_idx=None,
                   compensated=False):
    fx, zeta, area = _f(fx), _f(zeta), _f(area)
    mask = np.ascontiguousarray(mask, np.uint8)
    idx = None if tgt_idx is None else np.ascontiguousarray(tgt_idx, np.int64)
    n = fx.shape[0] if idx is None else idx.shape[0]
    psi = np.zeros(n) if want_psi else None
    u = np.zeros((n, 3)) if want_u else None
    lib().oracle_bve_face_solve(_p(psi), _p(u), n, _p(idx), _p(fx), _p(zeta), _p(area), _p(mask),
                                fx.shape[0], int(compensated))
    return psi, u


def ic2d_passive_sums(x, y, zeta, area, mask, eps, tgt_idx=None, compensated=False,
                      want_psi=True):
    """Incompressible2DPassiveSums: (u, psi); want_psi=False skips the
    stream function (psi is returned as None)."""
    x, y, zeta, area = _f(x), _f(y), _f(zeta), _f(area)
    ndim = x.shape[1]
    mask = np.ascontiguousarray(mask, np.uint8)
    idx = None if tgt_idx is None else np.ascontiguousarray(tgt_idx, np.int64)
    n = x.shape[0] if idx is None else idx.shape[0]
    u, psi = np.zeros((n, ndim)), (np.zeros(n) if want_psi else None)
    lib().oracle_ic2d_passive_sums(ndim, _p(u), _p(psi), _p(x), n, _p(idx), _p(y), _p(zeta),
                                   _p(area), _p(mask), float(eps), y.shape[0], int(compensated))
    return u, psi


def ic2d_active_sums(y, zeta, area, mask, eps, self_rule=0, tgt_idx=None, compensated=False):
    y, zeta, area = _f(y), _f(zeta), _f(area)
    ndim = y.shape[1]
    mask = np.ascontiguousarray(mask, np.uint8)
    idx = None if tgt_idx is None else np.ascontiguousarray(tgt_idx, np.int64)
    n = y.shape[0] if idx is None else idx.shape[0]
    u, psi = np.zeros((n, ndim)), np.zeros(n)
    lib().oracle_ic2d_active_sums(ndim, _p(u), _p(psi), n, _p(idx), _p(y), _p(zeta), _p(area),
                                  _p(mask), float(eps), y.shape[0], int(self_rule),
                                  int(compensated))
    return u, psi


class BVEState:
    """Host copy of a BVE state advanced by the oracle's BVERK4."""

    def __init__(self, vx, vzeta, vvel, fx, fzeta, fvel, farea, fmask):
        self.vx, self.vzeta, self.vvel = _f(vx).copy(), _f(vzeta).copy(), _f(vvel).copy()
        self.fx, self.fzeta, self.fvel = _f(fx).copy(), _f(fzeta).copy(), _f(fvel).copy()
        self.farea = _f(farea)
        self.fmask = np.ascontiguousarray(fmask, np.uint8)

    def step(self, dt, Omega, eps=0.0, fix_facevort3=False, reproject=False):
        lib().oracle_bve_rk4_step(self.vx.shape[0], _p(self.vx), _p(self.vzeta), _p(self.vvel),
                                  self.fx.shape[0], _p(self.fx), _p(self.fzeta), _p(self.fvel),
                                  _p(self.farea), _p(self.fmask), float(dt), float(Omega),
                                  float(eps), int(fix_facevort3), int(reproject))


class IC2DState:
    """Host copy of an incompressible2d state advanced by the oracle's RK2."""

    def __init__(self, vx, vzeta, fx, fzeta, farea, fmask, eps, cor, self_rule=0):
        self.ndim = np.asarray(vx).shape[1]
        self.vx, self.vzeta = _f(vx).copy(), _f(vzeta).copy()
        self.fx, self.fzeta = _f(fx).copy(), _f(fzeta).copy()
        self.farea = _f(farea)
        self.fmask = np.ascontiguousarray(fmask, np.uint8)
        self.eps, self.cor, self.self_rule = float(eps), float(cor), int(self_rule)
        nv, nf, nd = self.vx.shape[0], self.fx.shape[0], self.ndim
        self.vvel, self.vpsi = np.zeros((nv, nd)), np.zeros(nv)
        self.fvel, self.fpsi = np.zeros((nf, nd)), np.zeros(nf)

    def init_direct_sums(self):
        lib().oracle_ic2d_init_direct_sums(self.ndim, self.vx.shape[0], _p(self.vx), _p(self.vvel),
                                           _p(self.vpsi), self.fx.shape[0], _p(self.fx),
                                           _p(self.fzeta), _p(self.fvel), _p(self.fpsi),
                                           _p(self.farea), _p(self.fmask), self.eps,
                                           self.self_rule)

    def step(self, dt):
        lib().oracle_ic2d_rk2_step(self.ndim, self.vx.shape[0], _p(self.vx), _p(self.vzeta),
                                   _p(self.vvel), _p(self.vpsi), self.fx.shape[0], _p(self.fx),
                                   _p(self.fzeta), _p(self.fvel), _p(self.fpsi), _p(self.farea),
                                   _p(self.fmask), float(dt), self.eps, self.cor, self.self_rule)


def swe_plane_sums(tx, ts, y, zeta, sigma, area, mask, ss, eps, pse_eps, collocated=False):
    """Planar SWE sums (n x 9): u, v, du/dx, du/dy, dv/dx, dv/dy, lap(s), psi, phi."""
    tx, ts, y = _f(tx), _f(ts), _f(y)
    zeta, sigma, area, ss = _f(zeta), _f(sigma), _f(area), _f(ss)
    mask = np.ascontiguousarray(mask, np.uint8)
    out = np.zeros((tx.shape[0], 9))
    lib().oracle_swe_plane_sums(tx.shape[0], _p(tx), _p(ts), y.shape[0], _p(y), _p(zeta),
                                _p(sigma), _p(area), _p(mask), _p(ss), float(eps),
                                float(pse_eps), int(collocated), _p(out))
    return out


def swe_sphere_sums(tx, y, zeta, sigma, area, mask, eps, collocated=False):
    """Spherical SWE sums (n x 12): u, v, w and the velocity-gradient tensor
    (row-major) of SphereVertexSums / SphereFaceSums."""
    tx, y = _f(tx), _f(y)
    zeta, sigma, area = _f(zeta), _f(sigma), _f(area)
    mask = np.ascontiguousarray(mask, np.uint8)
    out = np.zeros((tx.shape[0], 12))
    lib().oracle_swe_sphere_sums(tx.shape[0], _p(tx), y.shape[0], _p(y), _p(zeta), _p(sigma),
                                 _p(area), _p(mask), float(eps), int(collocated), _p(out))
    return out


def double_dot(m9):
    """sum_ij M_ij M_ji in the functors' loop order (src/lpm_swe_kernels.hpp:777-782)."""
    m9 = np.asarray(m9, np.float64)
    out = np.zeros(m9.shape[0])
    for a in range(3):
        for b in range(3):
            out = out + m9[:, 3 * a + b] * m9[:, 3 * b + a]
    return out


def invariants(zeta, vel, area, mask):
    zeta, vel, area = _f(zeta), _f(vel), _f(area)
    mask = np.ascontiguousarray(mask, np.uint8)
    out = np.zeros(3)
    lib().oracle_invariants(vel.shape[1], zeta.shape[0], _p(zeta), _p(vel), _p(area), _p(mask),
                            _p(out))
    return tuple(out)


def err_norms(appx, exact, wt=None, mask=None):
    """ErrNorms: (l1, l2, linf) of vector magnitudes or scalars."""
    a = _f(appx)
    e = _f(exact)
    if a.ndim == 1:
        a, e = a.reshape(-1, 1), e.reshape(-1, 1)
    w = None if wt is None else _f(wt)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    out = np.zeros(3)
    lib().oracle_err_norms(a.shape[1], a.shape[0], _p(a), _p(e), _p(w), _p(m), _p(out))
    return tuple(out)


# ---- inputs: the reference's meshes and initial conditions -----------------
# Mesh kinds and initial-condition kinds (the same numbers as the library's
# LPM_MESH_* / LPM_IC_* constants).
MESH_ICOS_TRI, MESH_CUBED_SPHERE, MESH_QUAD_RECT = 1, 2, 3
IC_SOLID_BODY, IC_GAUSSIAN_SPHERE, IC_RH54, IC_DIPOLE_PAIR, IC_MULTI_GAUSSIAN = 1, 2, 3, 4, 5

# The reference's seed files, parsed by tests/golden/make_mesh_seeds.py.
SEED_FILE = HERE.parent / "tests" / "golden" / "mesh_seeds.npz"
_SEEDS = {MESH_ICOS_TRI: ("icos", 3, True), MESH_CUBED_SPHERE: ("cubed", 3, True),
          MESH_QUAD_RECT: ("quad", 2, False)}
_seed_cache = {}


def seed(kind):
    """(coordinates, edges, face vertices, face edges) of a reference seed."""
    if kind not in _seed_cache:
        name = _SEEDS[kind][0]
        with np.load(SEED_FILE) as z:
            _seed_cache[kind] = tuple(np.ascontiguousarray(z[f"{name}_{t}"]) for t in
                                      ("crds", "edges", "faceverts", "faceedges"))
    return _seed_cache[kind]


def mesh_sizes(kind, level):
    """(vertices, face slots) of a uniform mesh: n_vertices_at_tree_level and
    the sum of n_faces_at_tree_level over levels (src/mesh/lpm_mesh_seed.cpp:306-371)."""
    if kind == MESH_ICOS_TRI:
        return 2 + 10 * 4 ** level, sum(20 * 4 ** i for i in range(level + 1))
    if kind == MESH_CUBED_SPHERE:
        return 2 + 6 * 4 ** level, sum(6 * 4 ** i for i in range(level + 1))
    side = 3 + sum(2 ** i for i in range(1, level + 1))
    return side * side, sum(4 * 4 ** i for i in range(level + 1))


def mesh_build(kind, level, radius=1.0):
    """The reference's uniform mesh (tree_init from its seed file): vertex
    coordinates, face centres (all tree levels), areas, masks and face vertex
    lists."""
    crds, edges, fverts, fedges = seed(kind)
    ndim, sphere = _SEEDS[kind][1], _SEEDS[kind][2]
    nfv = fverts.shape[1]
    nv, nf = mesh_sizes(kind, level)
    vx, fx = np.zeros((nv, ndim)), np.zeros((nf, ndim))
    fa, fm = np.zeros(nf), np.zeros(nf, np.uint8)
    fv = np.zeros((nf, nfv), np.int64)
    nverts0 = crds.shape[0] - fverts.shape[0]  # seed rows: vertices, then face centres
    rc = lib().oracle_mesh_build(ndim, int(sphere), nfv, nverts0, edges.shape[0], fverts.shape[0],
                                 _p(_f(crds)), _p(edges), _p(fverts), _p(fedges), float(radius),
                                 int(level), nv, nf, _p(vx), _p(fx), _p(fa), _p(fm), _p(fv))
    if rc != 0:
        raise RuntimeError("oracle_mesh_build: size mismatch")
    return vx, fx, fa, fm, fv


def ic_eval(kind, params, x):
    """Initial relative vorticity at the rows of x (see oracle_ic_eval)."""
    x = _f(x)
    prm = np.ascontiguousarray(params, np.float64)
    out = np.zeros(x.shape[0])
    rc = lib().oracle_ic_eval(int(kind), _p(prm), prm.size, x.shape[1], x.shape[0], _p(x),
                              _p(out))
    if rc != 0:
        raise ValueError("oracle_ic_eval: unknown kind or too few parameters")
    return out


def mesh(kind, level, radius=1.0):
    """(vertices, face centres, areas, masks) of the reference's uniform mesh."""
    vx, fx, fa, fm, _ = mesh_build(kind, level, radius)
    return vx, fx, fa, fm

"""ctypes binding of the C ABI declared in include/lpm_gb300.h.

The shared library is built in-tree (``lpm_gb300/_lib/liblpm_gb300.so``) by
``lpm_gb300.build``.  There is no fallback: if the library is missing or no
GPU is visible, the calls that need it raise ``LpmError``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "liblpm_gb300.so"

LPM_OK = 0
LPM_ERR_ARG = -1
LPM_ERR_CUDA = -2
LPM_ERR_TIMEOUT = -3
LPM_ERR_ALLOC = -4
LPM_ERR_STATE = -5

FP64 = 64
FP32C = 32
FP64_CHORD = 65
FP64_EXACT = 66
PLANE = 2
SPHERE = 3

STEP_FIX_FACEVORT3 = 1
STEP_REPROJECT = 2
STEP_SKIP_MASKED_TARGETS = 4
STEP_SKIP_SELF_ALWAYS = 8
STEP_NO_GRAPH = 16
STEP_TIME_NBODY = 32

MESH_ICOS_TRI = 1
MESH_CUBED_SPHERE = 2
MESH_QUAD_RECT = 3

IC_SOLID_BODY = 1
IC_GAUSSIAN_SPHERE = 2
IC_RH54 = 3
IC_DIPOLE_PAIR = 4
IC_MULTI_GAUSSIAN = 5

# Every symbol include/lpm_gb300.h declares (checked by the CPU test-suite).
EXPORTS = [
    "lpm_context_create", "lpm_context_destroy", "lpm_context_set_stream",
    "lpm_context_set_precision", "lpm_context_synchronize",
    "lpm_context_kernel_launches", "lpm_last_error", "lpm_device_count",
    "lpm_bve_vertex_solve", "lpm_bve_vertex_stream_fn", "lpm_bve_vertex_velocity",
    "lpm_bve_face_solve", "lpm_bve_face_stream_fn", "lpm_bve_face_velocity",
    "lpm_bve_vorticity_tendency", "lpm_ic2d_passive_sums", "lpm_ic2d_active_sums",
    "lpm_ic2d_tendencies", "lpm_ic2d_invariants", "lpm_err_norms",
    "lpm_bve_rk4_create", "lpm_bve_rk4_destroy", "lpm_bve_rk4_advance_timestep",
    "lpm_ic2d_rk2_create", "lpm_ic2d_rk2_destroy", "lpm_ic2d_rk2_advance_timestep",
    "lpm_mesh_sizes", "lpm_mesh_build", "lpm_ic_eval", "lpm_measure_fma_peak",
    "lpm_bve_rk4_nbody_time", "lpm_ic2d_rk2_nbody_time", "lpm_bve_vertex_velocity_static",
    "lpm_ensemble_create", "lpm_ensemble_destroy", "lpm_ensemble_velocity",
    "lpm_ensemble_advance_timestep", "lpm_ensemble_info", "lpm_ensemble_nbody_time",
    "lpm_ensemble_set_chunk_len", "lpm_sphere_tangency",
    "lpm_farfield_create", "lpm_farfield_destroy", "lpm_farfield_velocity", "lpm_farfield_train",
    "lpm_farfield_set_network", "lpm_farfield_get_weights", "lpm_farfield_set_weights",
    "lpm_farfield_grad", "lpm_farfield_stats", "lpm_bve_rk4_set_farfield", "lpm_tc_selftest", "lpm_farfield_timing",
    "lpm_octree_stats", "lpm_mesh_build_device", "lpm_swe_plane_vertex_sums",
    "lpm_swe_plane_face_sums", "lpm_swe_sphere_vertex_sums", "lpm_swe_sphere_face_sums",
    "lpm_mesh_face_vertices", "lpm_vtk_write_polymesh", "lpm_bve_direct_sum",
    "lpm_plane_direct_sum", "lpm_bve_rk4_step", "lpm_ic2d_rk2_step", "lpm_ensemble_run",
    "lpm_one_call_release", "lpm_wait_selftest", "lpm_ensemble_shape", "lpm_ensemble_set_kernel",
    "lpm_netcdf_write_polymesh", "lpm_context_set_kernel_shape", "lpm_bve_rk4_kernel_shape",
]


class LpmError(RuntimeError):
    """Raised for a nonzero status from the library (std::runtime_error in C++)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"lpm error {code}: {msg}")
        self.code = code


class Crd3(C.Structure):
    """lpm_crd3: coordinate view with its count (one-call entry points)."""
    _fields_ = [("p", C.c_void_p), ("n", C.c_longlong), ("stride_i", C.c_longlong),
                ("stride_c", C.c_longlong)]


class View(C.Structure):
    _fields_ = [("p", C.c_void_p), ("stride_i", C.c_int64), ("stride_c", C.c_int64)]


_lib = None


def lib() -> C.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise LpmError(LPM_ERR_STATE,
                           f"{LIB_PATH} is missing: build it with python -m lpm_gb300.build")
        L = C.CDLL(str(LIB_PATH))
        _declare(L)
        _lib = L
    return _lib


def _declare(L: C.CDLL) -> None:
    vp, i64, i32, dbl, u32 = C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_uint32
    V = View
    sig = {
        "lpm_context_create": [C.POINTER(C.c_void_p), i32],
        "lpm_context_destroy": [vp],
        "lpm_context_set_stream": [vp, vp],
        "lpm_context_set_precision": [vp, i32],
        "lpm_context_set_kernel_shape": [vp, i32],
        "lpm_context_synchronize": [vp],
        "lpm_wait_selftest": [vp, i32],
        "lpm_context_kernel_launches": [vp],
        "lpm_last_error": [],
        "lpm_device_count": [],
        "lpm_bve_vertex_solve": [vp, vp, V, V, i64, V, vp, vp, vp, i64],
        "lpm_bve_vertex_stream_fn": [vp, vp, V, i64, V, vp, vp, vp, i64],
        "lpm_bve_vertex_velocity": [vp, V, V, i64, V, vp, vp, vp, i64],
        "lpm_bve_face_solve": [vp, vp, V, V, vp, vp, vp, i64],
        "lpm_bve_face_stream_fn": [vp, vp, V, vp, vp, vp, i64],
        "lpm_bve_face_velocity": [vp, V, V, vp, vp, vp, i64],
        "lpm_bve_vorticity_tendency": [vp, vp, V, i64, dbl, dbl],
        "lpm_ic2d_passive_sums": [vp, i32, V, vp, V, i64, V, vp, vp, vp, dbl, i64],
        "lpm_ic2d_active_sums": [vp, i32, V, vp, V, vp, vp, vp, dbl, i64, i32],
        "lpm_ic2d_tendencies": [vp, i32, vp, V, i64, dbl],
        "lpm_ic2d_invariants": [vp, i32, i64, vp, V, vp, vp, vp],
        "lpm_err_norms": [vp, i32, i64, V, V, vp, vp, vp],
        "lpm_bve_rk4_create": [vp, C.POINTER(C.c_void_p), i64, i64, dbl, dbl, dbl, i32, u32],
        "lpm_bve_rk4_destroy": [vp],
        "lpm_bve_rk4_advance_timestep": [vp, V, vp, V, V, vp, V, vp, vp],
        "lpm_ic2d_rk2_create": [vp, C.POINTER(C.c_void_p), i32, i64, i64, dbl, dbl, dbl, i32, u32],
        "lpm_ic2d_rk2_destroy": [vp],
        "lpm_ic2d_rk2_advance_timestep": [vp, V, vp, V, vp, V, vp, V, vp, vp, vp],
        "lpm_mesh_sizes": [i32, i32, C.POINTER(i64), C.POINTER(i64)],
        "lpm_mesh_build": [i32, i32, dbl, vp, vp, vp, vp],
        "lpm_ic_eval": [i32, vp, i32, i32, i64, vp, vp],
        "lpm_measure_fma_peak": [vp, i32, C.POINTER(dbl)],
        "lpm_bve_rk4_nbody_time": [vp, C.POINTER(dbl), C.POINTER(i64)],
        "lpm_bve_rk4_kernel_shape": [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)],
        "lpm_ic2d_rk2_nbody_time": [vp, C.POINTER(dbl), C.POINTER(i64)],
        "lpm_bve_vertex_velocity_static": [V, V, i64, V, vp, vp, vp, i64, vp],
        "lpm_ensemble_create": [vp, C.POINTER(C.c_void_p), i32, vp, vp, vp, dbl, dbl, dbl, i32,
                                u32],
        "lpm_ensemble_destroy": [vp],
        "lpm_ensemble_velocity": [vp, V, V, V, vp, V, vp],
        "lpm_ensemble_advance_timestep": [vp, V, vp, V, V, vp, V, vp],
        "lpm_ensemble_info": [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)],
        "lpm_ensemble_shape": [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)],
        "lpm_ensemble_set_kernel": [vp, i32, i32],
        "lpm_ensemble_nbody_time": [vp, C.POINTER(dbl), C.POINTER(i64)],
        "lpm_ensemble_set_chunk_len": [vp, i64],
        "lpm_sphere_tangency": [vp, vp, V, V, i64],
        "lpm_farfield_create": [vp, C.POINTER(C.c_void_p), dbl, i32, dbl],
        "lpm_farfield_destroy": [vp],
        "lpm_farfield_velocity": [vp, V, V, i64, V, vp, vp, vp, i64, dbl],
        "lpm_farfield_train": [vp, i64, i32, i32, dbl, C.c_uint64, i32, i32, dbl, vp],
        "lpm_farfield_set_network": [vp, i32],
        "lpm_farfield_get_weights": [vp, vp, vp],
        "lpm_farfield_set_weights": [vp, vp, vp],
        "lpm_farfield_grad": [vp, vp, vp, i32, vp],
        "lpm_farfield_stats": [vp, vp],
        "lpm_bve_rk4_set_farfield": [vp, vp, i32],
        "lpm_tc_selftest": [vp, vp, vp, vp, i32, i32, i32, i32],
        "lpm_farfield_timing": [vp, i32, C.POINTER(dbl), C.POINTER(dbl), C.POINTER(i64)],
        "lpm_octree_stats": [vp, i64, vp, i64, i32, vp],
        "lpm_mesh_build_device": [vp, i32, i32, dbl, vp, vp, vp, vp],
        "lpm_swe_plane_vertex_sums": [vp, V, vp, vp, vp, vp, vp, vp, vp, vp, V, vp, i64, V, vp, vp,
                                      vp, vp, vp, i64, dbl, dbl, i32],
        "lpm_swe_plane_face_sums": [vp, V, vp, vp, vp, vp, vp, vp, vp, vp, V, vp, vp, vp, vp, vp,
                                    i64, dbl, dbl, i32],
        "lpm_swe_sphere_vertex_sums": [vp, V, vp, vp, V, i64, V, vp, vp, vp, vp, i64, dbl, i32],
        "lpm_swe_sphere_face_sums": [vp, V, vp, vp, V, vp, vp, vp, vp, i64, dbl, i32],
        "lpm_mesh_face_vertices": [i32, i32, dbl, C.POINTER(i32), vp],
        "lpm_bve_direct_sum": [Crd3, Crd3, vp, vp, vp, C.c_longlong, i32, dbl, i32, i32, vp,
                               C.c_longlong, C.c_longlong, vp, vp],
        "lpm_plane_direct_sum": [Crd3, Crd3, vp, vp, vp, C.c_longlong, i32, dbl, i32, i32, vp,
                                 C.c_longlong, C.c_longlong, vp, vp],
        "lpm_bve_rk4_step": [vp, V, vp, V, V, vp, V, vp, vp],
        "lpm_ic2d_rk2_step": [vp, V, vp, V, vp, V, vp, V, vp, vp, vp],
        "lpm_ensemble_run": [vp, i32, V, vp, V, V, vp, V, vp],
        "lpm_one_call_release": [],
        "lpm_vtk_write_polymesh": [C.c_char_p, i32, i64, vp, vp, i64, i32, vp, vp, vp, i32, vp],
        "lpm_netcdf_write_polymesh": [C.c_char_p, i32, i64, vp, i64, i32, vp, vp, vp, vp, dbl,
                                      i32, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.lpm_last_error.restype = C.c_char_p
    L.lpm_context_kernel_launches.restype = C.c_int64


def check(code: int) -> None:
    if code != LPM_OK:
        raise LpmError(code, lib().lpm_last_error().decode())


def ptr(t) -> int | None:
    """Device (or host numpy) address of a tensor/array, None for None."""
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def crd3(t) -> Crd3:
    """lpm_crd3 of a 2-D torch tensor (rows = points), any strides."""
    if t.dim() != 2:
        raise ValueError("coordinate views must be 2-D (n x ndim)")
    return Crd3(t.data_ptr(), t.shape[0], t.stride(0), t.stride(1))


def view(t) -> View:
    """lpm_view of a 2-D torch tensor (rows = points), any strides."""
    if t is None:
        return View(None, 0, 0)
    if t.dim() != 2:
        raise ValueError("coordinate/vector views must be 2-D (n x ndim)")
    return View(t.data_ptr(), t.stride(0), t.stride(1))


class Context:
    """Owns an lpm_context bound to one device and a CUDA stream."""

    def __init__(self, device: int = 0, precision: int = FP64, stream=None):
        self._h = C.c_void_p()
        check(lib().lpm_context_create(C.byref(self._h), device))
        self.device = device
        self.set_precision(precision)
        if stream is not None:
            self.set_stream(stream)

    @property
    def handle(self):
        return self._h

    def set_precision(self, precision: int) -> None:
        check(lib().lpm_context_set_precision(self._h, precision))
        self.precision = precision

    def set_kernel_shape(self, shape: int) -> None:
        """Fixes the FP32 N-body kernel shape (0-5) of later LPM_FP32C sums,
        or -1 for per-size autotuning (the default)."""
        check(lib().lpm_context_set_kernel_shape(self._h, int(shape)))

    def set_stream(self, stream) -> None:
        """stream: a torch.cuda.Stream, or an integer cudaStream_t."""
        raw = getattr(stream, "cuda_stream", stream)
        check(lib().lpm_context_set_stream(self._h, C.c_void_p(int(raw))))

    def synchronize(self) -> None:
        check(lib().lpm_context_synchronize(self._h))

    @property
    def kernel_launches(self) -> int:
        return int(lib().lpm_context_kernel_launches(self._h))

    def fma_peak_tflops(self, precision: int) -> float:
        out = C.c_double()
        check(lib().lpm_measure_fma_peak(self._h, precision, C.byref(out)))
        return out.value

    def close(self) -> None:
        if self._h:
            lib().lpm_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    if device not in _default_ctx:
        _default_ctx[device] = Context(device)
    return _default_ctx[device]


# ---- host-side inputs -----------------------------------------------------

def mesh_sizes(kind: int, level: int) -> tuple[int, int]:
    nv, nf = C.c_int64(), C.c_int64()
    check(lib().lpm_mesh_sizes(kind, level, C.byref(nv), C.byref(nf)))
    return nv.value, nf.value


def build_mesh(kind: int, level: int, radius: float = 1.0):
    """Uniform panel mesh: (vx[nv, ndim], fx[nf, ndim], farea[nf], fmask[nf])."""
    nv, nf = mesh_sizes(kind, level)
    ndim = 2 if kind == MESH_QUAD_RECT else 3
    vx = np.empty((nv, ndim), np.float64)
    fx = np.empty((nf, ndim), np.float64)
    fa = np.empty(nf, np.float64)
    fm = np.empty(nf, np.uint8)
    check(lib().lpm_mesh_build(kind, level, radius, ptr(vx), ptr(fx), ptr(fa), ptr(fm)))
    return vx, fx, fa, fm


def mesh_face_vertices(kind: int, level: int, radius: float = 1.0) -> np.ndarray:
    """Face vertex lists (nf x nfv, int32) of the mesh build_mesh makes."""
    nfv = C.c_int32()
    check(lib().lpm_mesh_face_vertices(kind, level, radius, C.byref(nfv), None))
    _, nf = mesh_sizes(kind, level)
    out = np.empty((nf, nfv.value), np.int32)
    check(lib().lpm_mesh_face_vertices(kind, level, radius, C.byref(nfv), ptr(out)))
    return out


def build_mesh_device(ctx, kind: int, level: int, radius: float = 1.0):
    """The same mesh built on the context's GPU: torch tensors (vx, fx, farea, fmask)."""
    import torch

    nv, nf = mesh_sizes(kind, level)
    ndim = 2 if kind == MESH_QUAD_RECT else 3
    dev = torch.device("cuda", ctx.device)
    vx = torch.empty((nv, ndim), dtype=torch.float64, device=dev)
    fx = torch.empty((nf, ndim), dtype=torch.float64, device=dev)
    fa = torch.empty(nf, dtype=torch.float64, device=dev)
    fm = torch.empty(nf, dtype=torch.uint8, device=dev)
    check(lib().lpm_mesh_build_device(ctx.handle, kind, level, radius, vx.data_ptr(),
                                      fx.data_ptr(), fa.data_ptr(), fm.data_ptr()))
    return vx, fx, fa, fm


def eval_ic(kind: int, params, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float64)
    p = np.ascontiguousarray(np.asarray(params, np.float64).ravel())
    out = np.empty(x.shape[0], np.float64)
    check(lib().lpm_ic_eval(kind, ptr(p) if p.size else None, p.size, x.shape[1],
                            x.shape[0], ptr(x), ptr(out)))
    return out

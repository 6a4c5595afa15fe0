// capi.cu -- the extern "C" boundary (include/lpm_gb300.h): argument
// validation, context lifetime, error reporting and dispatch of the functor
// entry points onto lpm::direct_sum.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "lpm_host.hpp"
#include "nbody.cuh"

namespace lpm {

namespace {
thread_local std::string g_last_error;
}  // namespace

int fail(int code, const char* msg) {
  g_last_error = msg;
  return code;
}

int handle_exception() {
  try {
    throw;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return LPM_ERR_ALLOC;
  } catch (const std::invalid_argument& e) {
    g_last_error = e.what();
    return LPM_ERR_ARG;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return LPM_ERR_STATE;
  } catch (...) {
    g_last_error = "unknown error";
    return LPM_ERR_STATE;
  }
}

void Arena::reserve(size_t bytes) {
  if (bytes <= cap) return;
  if (fixed)
    throw Error(LPM_ERR_ARG, "this call needs " + std::to_string(bytes) +
                                 " bytes of scratch; the fixed scratch holds " +
                                 std::to_string(cap));
  if (base) {
    cudaDeviceSynchronize();
    cudaFree(base);
    base = nullptr;
    cap = 0;
  }
  size_t want = bytes + bytes / 4 + (size_t(1) << 20);
  void* p = nullptr;
  const cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(LPM_ERR_ALLOC, std::string("device scratch allocation of ") +
                                   std::to_string(want) + " bytes failed: " +
                                   cudaGetErrorString(e));
  }
  base = static_cast<char*>(p);
  cap = want;
  off = 0;
}

void Arena::release() {
  if (base) cudaFree(base);
  base = nullptr;
  cap = off = 0;
}

void check_device_error(lpm_context& ctx) {
  int h = 0;
  LPM_CUDA(cudaMemcpyAsync(&h, ctx.d_err, sizeof(int), cudaMemcpyDeviceToHost,
                           ctx.stream));
  LPM_CUDA(cudaStreamSynchronize(ctx.stream));
  if (h) {
    LPM_CUDA(cudaMemsetAsync(ctx.d_err, 0, sizeof(int), ctx.stream));
    throw Error(LPM_ERR_TIMEOUT,
                "a bounded device-side wait gave up (tile copy did not "
                "complete); results of the affected calls are invalid");
  }
}

}  // namespace lpm

namespace {

using lpm::fail;

// Indices are 32-bit inside the kernels.
bool bad_count(int64_t n) { return n < 0 || n > (int64_t(1) << 31) - 1; }

int check_view(const lpm_view& v, int64_t n, const char* what, bool nullable) {
  if (n == 0) return LPM_OK;
  if (!v.p) {
    if (nullable) return LPM_OK;
    std::string m = std::string(what) + ": null pointer";
    return fail(LPM_ERR_ARG, m.c_str());
  }
  if (v.stride_i == 0 && n > 1) {
    std::string m = std::string(what) + ": zero row stride";
    return fail(LPM_ERR_ARG, m.c_str());
  }
  return LPM_OK;
}

int check_ctx(lpm_context* ctx) {
  if (!ctx) return fail(LPM_ERR_ARG, "null context");
  return LPM_OK;
}

int check_sources(lpm_view fx, const double* zeta, const double* area,
                  const uint8_t* mask, int64_t nf) {
  if (bad_count(nf)) return fail(LPM_ERR_ARG, "source count out of range [0, 2^31-1]");
  if (nf > 0 && (!zeta || !area || !mask))
    return fail(LPM_ERR_ARG, "null source vorticity, area or mask");
  return check_view(fx, nf, "source coordinates", false);
}

lpm::SrcSpec srcspec(lpm_view fx, const double* zeta, const double* area,
                     const uint8_t* mask, int64_t nf) {
  return lpm::SrcSpec{lpm::to_view(fx), zeta, area, mask, nf};
}

lpm::TgtSeg seg(lpm_view x, int64_t n, lpm_view u, double* psi, bool coll) {
  return lpm::TgtSeg{lpm::to_view(x), n, lpm::to_view(u), psi, coll};
}

// BVE functors: eps = 0, the reference biot_savart / greens_fn arithmetic.
int bve_sum(lpm_context* ctx, double* psi, lpm_view u, lpm_view tx,
            int64_t nt, bool collocated, lpm_view fx, const double* zeta,
            const double* area, const uint8_t* mask, int64_t nf, bool wu,
            bool wp) {
  if (int r = check_ctx(ctx)) return r;
  lpm::DeviceGuard device_guard(ctx->device);
  if (int r = check_sources(fx, zeta, area, mask, nf)) return r;
  if (bad_count(nt)) return fail(LPM_ERR_ARG, "target count out of range");
  if (int r = check_view(tx, nt, "target coordinates", false)) return r;
  if (wu)
    if (int r = check_view(u, nt, "velocity output", false)) return r;
  if (wp && nt > 0 && !psi) return fail(LPM_ERR_ARG, "null stream-function output");
  if (!wu && !wp) return LPM_OK;
  lpm::SumSpec s{3, lpm::FORM_BVE, ctx->precision, 0.0, wu, wp, true};
  const lpm::SrcSpec src = srcspec(fx, zeta, area, mask, nf);
  const lpm::TgtSeg g = seg(tx, nt, u, psi, collocated);
  lpm::direct_sum(*ctx, s, src, &g, 1);
  return LPM_OK;
}

}  // namespace

extern "C" {

const char* lpm_last_error(void) { return lpm::g_last_error.c_str(); }

int lpm_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int lpm_context_create(lpm_context** out, int device) {
  try {
    if (!out) return fail(LPM_ERR_ARG, "lpm_context_create: null output");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
      cudaGetLastError();
      return fail(LPM_ERR_CUDA, "lpm_context_create: no CUDA device is visible");
    }
    if (device < 0 || device >= n) return fail(LPM_ERR_ARG, "lpm_context_create: bad device id");
    lpm::DeviceGuard device_guard(device);
    LPM_CUDA(device_guard.status);
    auto* c = new lpm_context();
    c->device = device;
    cudaDeviceProp prop;
    LPM_CUDA(cudaGetDeviceProperties(&prop, device));
    c->num_sms = prop.multiProcessorCount;
    LPM_CUDA(cudaMalloc(&c->d_err, sizeof(int)));
    LPM_CUDA(cudaMemset(c->d_err, 0, sizeof(int)));
    *out = c;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_context_destroy(lpm_context* ctx) {
  if (!ctx) return LPM_OK;
  lpm::DeviceGuard device_guard(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->arena.release();
  if (ctx->d_err) cudaFree(ctx->d_err);
  delete ctx;
  return LPM_OK;
}

int lpm_context_set_stream(lpm_context* ctx, void* stream) {
  if (!ctx) return fail(LPM_ERR_ARG, "null context");
  ctx->stream = static_cast<cudaStream_t>(stream);
  return LPM_OK;
}

int lpm_context_set_precision(lpm_context* ctx, int precision) {
  if (!ctx) return fail(LPM_ERR_ARG, "null context");
  if (precision != LPM_FP64 && precision != LPM_FP32C && precision != LPM_FP64_CHORD &&
      precision != LPM_FP64_EXACT)
    return fail(LPM_ERR_ARG,
                "precision must be LPM_FP64 (64), LPM_FP64_CHORD (65), LPM_FP64_EXACT (66) "
                "or LPM_FP32C (32)");
  ctx->precision = precision;
  return LPM_OK;
}

int lpm_context_set_kernel_shape(lpm_context* ctx, int shape) {
  if (!ctx) return fail(LPM_ERR_ARG, "null context");
  if (shape < -1 || shape >= lpm::kNumF32Shapes)
    return fail(LPM_ERR_ARG, ("lpm_context_set_kernel_shape: shape must be -1 (autotune) or 0-" +
                              std::to_string(lpm::kNumF32Shapes - 1))
                                 .c_str());
  ctx->forced_shape = shape;
  return LPM_OK;
}

int lpm_context_synchronize(lpm_context* ctx) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    lpm::check_device_error(*ctx);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int64_t lpm_context_kernel_launches(const lpm_context* ctx) {
  return ctx ? ctx->launches : -1;
}

int lpm_bve_vertex_solve(lpm_context* ctx, double* psi, lpm_view u,
                         lpm_view vx, int64_t nverts, lpm_view fx,
                         const double* zeta, const double* area,
                         const uint8_t* mask, int64_t nfaces) {
  try {
    return bve_sum(ctx, psi, u, vx, nverts, false, fx, zeta, area, mask, nfaces,
                   u.p != nullptr, psi != nullptr);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_vertex_stream_fn(lpm_context* ctx, double* psi, lpm_view vx,
                             int64_t nverts, lpm_view fx, const double* zeta,
                             const double* area, const uint8_t* mask,
                             int64_t nfaces) {
  try {
    if (nverts > 0 && !psi) return fail(LPM_ERR_ARG, "null stream-function output");
    return bve_sum(ctx, psi, lpm_view{nullptr, 0, 0}, vx, nverts, false, fx,
                   zeta, area, mask, nfaces, false, true);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_vertex_velocity(lpm_context* ctx, lpm_view u, lpm_view vx,
                            int64_t nverts, lpm_view fx, const double* zeta,
                            const double* area, const uint8_t* mask,
                            int64_t nfaces) {
  try {
    if (nverts > 0 && !u.p) return fail(LPM_ERR_ARG, "null velocity output");
    return bve_sum(ctx, nullptr, u, vx, nverts, false, fx, zeta, area, mask,
                   nfaces, true, false);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_face_solve(lpm_context* ctx, double* psi, lpm_view u, lpm_view fx,
                       const double* zeta, const double* area,
                       const uint8_t* mask, int64_t nfaces) {
  try {
    return bve_sum(ctx, psi, u, fx, nfaces, true, fx, zeta, area, mask, nfaces,
                   u.p != nullptr, psi != nullptr);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_face_stream_fn(lpm_context* ctx, double* psi, lpm_view fx,
                           const double* zeta, const double* area,
                           const uint8_t* mask, int64_t nfaces) {
  try {
    if (nfaces > 0 && !psi) return fail(LPM_ERR_ARG, "null stream-function output");
    return bve_sum(ctx, psi, lpm_view{nullptr, 0, 0}, fx, nfaces, true, fx, zeta,
                   area, mask, nfaces, false, true);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_face_velocity(lpm_context* ctx, lpm_view u, lpm_view fx,
                          const double* zeta, const double* area,
                          const uint8_t* mask, int64_t nfaces) {
  try {
    if (nfaces > 0 && !u.p) return fail(LPM_ERR_ARG, "null velocity output");
    return bve_sum(ctx, nullptr, u, fx, nfaces, true, fx, zeta, area, mask,
                   nfaces, true, false);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_vorticity_tendency(lpm_context* ctx, double* dzeta, lpm_view u,
                               int64_t n, double dt, double Omega) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (bad_count(n)) return fail(LPM_ERR_ARG, "count out of range");
    if (n > 0 && !dzeta) return fail(LPM_ERR_ARG, "null output");
    if (int r = check_view(u, n, "velocity", false)) return r;
    lpm::bve_tendency(*ctx, dzeta, lpm::to_view(u), n, dt, Omega);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ic2d_passive_sums(lpm_context* ctx, int ndim, lpm_view u, double* psi,
                          lpm_view x, int64_t n_passive, lpm_view y,
                          const double* zeta, const double* area,
                          const uint8_t* mask, double eps, int64_t n_active) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (ndim != LPM_SPHERE && ndim != LPM_PLANE) return fail(LPM_ERR_ARG, "ndim must be 2 or 3");
    if (!std::isfinite(eps) || eps < 0) return fail(LPM_ERR_ARG, "eps must be finite and >= 0");
    if (int r = check_sources(y, zeta, area, mask, n_active)) return r;
    if (bad_count(n_passive)) return fail(LPM_ERR_ARG, "target count out of range");
    if (int r = check_view(x, n_passive, "target coordinates", false)) return r;
    const bool wu = u.p != nullptr, wp = psi != nullptr;
    if (!wu && !wp) return LPM_OK;
    lpm::SumSpec s{ndim, ndim == 3 ? lpm::FORM_SPHERE : lpm::FORM_PLANE,
                   ctx->precision, eps, wu, wp, false};
    const lpm::SrcSpec src = srcspec(y, zeta, area, mask, n_active);
    const lpm::TgtSeg g = seg(x, n_passive, u, psi, false);
    lpm::direct_sum(*ctx, s, src, &g, 1);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ic2d_active_sums(lpm_context* ctx, int ndim, lpm_view u, double* psi,
                         lpm_view xy, const double* zeta, const double* area,
                         const uint8_t* mask, double eps, int64_t n_active,
                         int self_rule) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (ndim != LPM_SPHERE && ndim != LPM_PLANE) return fail(LPM_ERR_ARG, "ndim must be 2 or 3");
    if (!std::isfinite(eps) || eps < 0) return fail(LPM_ERR_ARG, "eps must be finite and >= 0");
    if (self_rule != 0 && self_rule != 1) return fail(LPM_ERR_ARG, "self_rule must be 0 or 1");
    if (int r = check_sources(xy, zeta, area, mask, n_active)) return r;
    const bool wu = u.p != nullptr, wp = psi != nullptr;
    if (!wu && !wp) return LPM_OK;
    // FloatingPoint<Real>::zero(eps): |eps| < machine epsilon
    const bool skip = self_rule == 1 || std::fabs(eps) < 2.220446049250313e-16;
    lpm::SumSpec s{ndim, ndim == 3 ? lpm::FORM_SPHERE : lpm::FORM_PLANE,
                   ctx->precision, eps, wu, wp, skip};
    const lpm::SrcSpec src = srcspec(xy, zeta, area, mask, n_active);
    const lpm::TgtSeg g = seg(xy, n_active, u, psi, true);
    lpm::direct_sum(*ctx, s, src, &g, 1);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ic2d_tendencies(lpm_context* ctx, int ndim, double* dzeta, lpm_view u,
                        int64_t n, double cor) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (ndim != LPM_SPHERE && ndim != LPM_PLANE) return fail(LPM_ERR_ARG, "ndim must be 2 or 3");
    if (bad_count(n)) return fail(LPM_ERR_ARG, "count out of range");
    if (n > 0 && !dzeta) return fail(LPM_ERR_ARG, "null output");
    if (int r = check_view(u, n, "velocity", false)) return r;
    lpm::ic2d_tendency(*ctx, ndim, dzeta, lpm::to_view(u), n, cor);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_sphere_tangency(lpm_context* ctx, double* udotx, lpm_view x, lpm_view u,
                        int64_t n) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (bad_count(n)) return fail(LPM_ERR_ARG, "count out of range");
    if (n > 0 && !udotx) return fail(LPM_ERR_ARG, "null output");
    if (int r = check_view(x, n, "positions", false)) return r;
    if (int r = check_view(u, n, "velocity", false)) return r;
    lpm::tangency(*ctx, udotx, lpm::to_view(x), lpm::to_view(u), n);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ic2d_invariants(lpm_context* ctx, int ndim, int64_t nfaces,
                        const double* zeta, lpm_view vel, const double* area,
                        const uint8_t* mask, double out[3]) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (ndim != LPM_SPHERE && ndim != LPM_PLANE) return fail(LPM_ERR_ARG, "ndim must be 2 or 3");
    if (!out) return fail(LPM_ERR_ARG, "null output");
    if (bad_count(nfaces)) return fail(LPM_ERR_ARG, "count out of range");
    if (nfaces > 0 && (!zeta || !area || !mask)) return fail(LPM_ERR_ARG, "null input array");
    if (int r = check_view(vel, nfaces, "velocity", false)) return r;
    lpm::invariants(*ctx, ndim, nfaces, zeta, lpm::to_view(vel), area, mask, out);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_err_norms(lpm_context* ctx, int ndim, int64_t n, lpm_view appx,
                  lpm_view exact, const double* wt, const uint8_t* mask,
                  double out[3]) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (ndim < 1 || ndim > 3) return fail(LPM_ERR_ARG, "ndim must be 1, 2 or 3");
    if (!out) return fail(LPM_ERR_ARG, "null output");
    if (bad_count(n)) return fail(LPM_ERR_ARG, "count out of range");
    if (int r = check_view(appx, n, "approximation", false)) return r;
    if (int r = check_view(exact, n, "exact", false)) return r;
    lpm::err_norms(*ctx, ndim, n, lpm::to_view(appx), lpm::to_view(exact), wt,
                   mask, out);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_mesh_sizes(int kind, int level, int64_t* nverts, int64_t* nfaces) {
  try {
    if (!nverts || !nfaces) return fail(LPM_ERR_ARG, "null output");
    lpm::mesh_sizes(kind, level, nverts, nfaces);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_mesh_build(int kind, int level, double radius, double* vx, double* fx,
                   double* farea, uint8_t* fmask) {
  try {
    if (!vx || !fx || !farea || !fmask) return fail(LPM_ERR_ARG, "null output array");
    if (!(radius > 0) || !std::isfinite(radius)) return fail(LPM_ERR_ARG, "radius must be > 0");
    lpm::mesh_build(kind, level, radius, vx, fx, farea, fmask);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ic_eval(int kind, const double* params, int nparams, int ndim,
                int64_t n, const double* x, double* zeta) {
  try {
    if (n > 0 && (!x || !zeta)) return fail(LPM_ERR_ARG, "null array");
    if (nparams > 0 && !params) return fail(LPM_ERR_ARG, "null params");
    lpm::ic_eval(kind, params, nparams, ndim, n, x, zeta);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_wait_selftest(lpm_context* ctx, int spin_limit) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (spin_limit < 1 || spin_limit > (1 << 20))
      return fail(LPM_ERR_ARG, "lpm_wait_selftest: spin_limit must be in [1, 2^20]");
    lpm::wait_selftest(*ctx, unsigned(spin_limit));
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_measure_fma_peak(lpm_context* ctx, int precision, double* tflops) {
  try {
    if (int r = check_ctx(ctx)) return r;
    lpm::DeviceGuard device_guard(ctx->device);
    if (!tflops) return fail(LPM_ERR_ARG, "null output");
    if (precision != LPM_FP64 && precision != LPM_FP32C)
      return fail(LPM_ERR_ARG, "bad precision");
    *tflops = lpm::fma_peak(*ctx, precision);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

}  // extern "C"

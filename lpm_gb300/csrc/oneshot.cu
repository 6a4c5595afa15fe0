// oneshot.cu -- one-call forms of the boundary for hosts that do not keep an
// lpm_context: a direct sum given coordinate views, a precision and a CUDA
// stream, and step/run forms of the steppers and the ensemble.
//
// The direct-sum calls use a context cached per host thread and device,
// created on first use and freed by lpm_one_call_release (its scratch memory
// can be large: the FP64 chunk partials of the last call).  Calls are
// stream-ordered on the stream they are given; when a thread switches
// streams, the previous stream is synchronised first, because the context's
// scratch memory is reused by the next call.
#include <cmath>

#include <cuda_runtime.h>

#include "lpm_host.hpp"

namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu
}  // namespace lpm

namespace {

constexpr int kMaxDevices = 64;
thread_local lpm_context* t_ctx[kMaxDevices] = {};

int thread_context(void* stream, int precision, lpm_context** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return lpm::fail(LPM_ERR_CUDA, "no current CUDA device");
  }
  if (!t_ctx[dev])
    if (int r = lpm_context_create(&t_ctx[dev], dev)) return r;
  lpm_context* c = t_ctx[dev];
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (c->stream != s) {
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
      cudaGetLastError();
      return lpm::fail(LPM_ERR_CUDA, "synchronising the previous stream failed");
    }
    c->stream = s;
  }
  if (int r = lpm_context_set_precision(c, precision)) return r;
  *out = c;
  return LPM_OK;
}

lpm_view view3(const lpm_crd3& v) { return lpm_view{const_cast<double*>(v.p), v.stride_i, v.stride_c}; }

int direct_sum(int ndim, lpm_crd3 tgt, lpm_crd3 src, const double* zeta, const double* area,
               const unsigned char* mask, long long n_src, int collocated, double eps, int want,
               int precision, double* u_out, long long u_stride_i, long long u_stride_c,
               double* psi_out, void* stream) {
  if (want < 1 || want > 3) return lpm::fail(LPM_ERR_ARG, "want must be 1 (u), 2 (psi) or 3");
  if (!(eps >= 0) || !std::isfinite(eps)) return lpm::fail(LPM_ERR_ARG, "eps must be finite and >= 0");
  if (collocated && (tgt.p != src.p || tgt.n != n_src || tgt.stride_i != src.stride_i ||
                     tgt.stride_c != src.stride_c))
    return lpm::fail(LPM_ERR_ARG, "collocated: the target view must be the source view");
  lpm_context* ctx = nullptr;
  if (int r = thread_context(stream, precision, &ctx)) return r;
  const lpm_view u = (want & 1) ? lpm_view{u_out, u_stride_i, u_stride_c} : lpm_view{nullptr, 0, 0};
  double* psi = (want & 2) ? psi_out : nullptr;
  if ((want & 1) && tgt.n > 0 && !u_out) return lpm::fail(LPM_ERR_ARG, "null velocity output");
  if ((want & 2) && tgt.n > 0 && !psi_out) return lpm::fail(LPM_ERR_ARG, "null stream-function output");
  if (ndim == 3 && eps == 0) {
    // the BVE functors (biot_savart / greens_fn); collocated targets skip i == j
    return collocated ? lpm_bve_face_solve(ctx, psi, u, view3(src), zeta, area, mask, n_src)
                      : lpm_bve_vertex_solve(ctx, psi, u, view3(tgt), tgt.n, view3(src), zeta,
                                             area, mask, n_src);
  }
  // the smoothed kernels of Incompressible2DKernels; on the sphere the
  // collocated rule stays the BVE one (skip i == j), in the plane it is the
  // incompressible-2D one (skip i == j only when eps is zero)
  if (collocated)
    return lpm_ic2d_active_sums(ctx, ndim, u, psi, view3(src), zeta, area, mask, eps, n_src,
                                ndim == 3 ? 1 : 0);
  return lpm_ic2d_passive_sums(ctx, ndim, u, psi, view3(tgt), tgt.n, view3(src), zeta, area,
                               mask, eps, n_src);
}

}  // namespace

extern "C" {

int lpm_bve_direct_sum(lpm_crd3 tgt, lpm_crd3 src, const double* zeta, const double* area,
                       const unsigned char* mask, long long n_src, int collocated, double eps,
                       int want, int precision, double* u_out, long long u_stride_i,
                       long long u_stride_c, double* psi_out, void* cuda_stream) {
  try {
    return direct_sum(3, tgt, src, zeta, area, mask, n_src, collocated, eps, want, precision,
                      u_out, u_stride_i, u_stride_c, psi_out, cuda_stream);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_plane_direct_sum(lpm_crd3 tgt, lpm_crd3 src, const double* zeta, const double* area,
                         const unsigned char* mask, long long n_src, int collocated, double eps,
                         int want, int precision, double* u_out, long long u_stride_i,
                         long long u_stride_c, double* psi_out, void* cuda_stream) {
  try {
    return direct_sum(2, tgt, src, zeta, area, mask, n_src, collocated, eps, want, precision,
                      u_out, u_stride_i, u_stride_c, psi_out, cuda_stream);
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_one_call_release(void) {
  int status = LPM_OK;
  for (int d = 0; d < kMaxDevices; ++d) {
    if (!t_ctx[d]) continue;
    if (int r = lpm_context_destroy(t_ctx[d])) status = r;
    t_ctx[d] = nullptr;
  }
  return status;
}

int lpm_bve_rk4_step(lpm_bve_rk4* st, lpm_view vx, double* vzeta, lpm_view vvel, lpm_view fx,
                     double* fzeta, lpm_view fvel, const double* farea, const uint8_t* fmask) {
  return lpm_bve_rk4_advance_timestep(st, vx, vzeta, vvel, fx, fzeta, fvel, farea, fmask);
}

int lpm_ic2d_rk2_step(lpm_ic2d_rk2* st, lpm_view vx, double* vzeta, lpm_view vvel, double* vpsi,
                      lpm_view fx, double* fzeta, lpm_view fvel, double* fpsi,
                      const double* farea, const uint8_t* fmask) {
  return lpm_ic2d_rk2_advance_timestep(st, vx, vzeta, vvel, vpsi, fx, fzeta, fvel, fpsi, farea,
                                       fmask);
}

int lpm_ensemble_run(lpm_ensemble* e, int nsteps, lpm_view vx, double* vzeta, lpm_view vvel,
                     lpm_view fx, double* fzeta, lpm_view fvel, const double* farea) {
  if (nsteps < 0) return lpm::fail(LPM_ERR_ARG, "nsteps must be >= 0");
  for (int k = 0; k < nsteps; ++k)
    if (int r = lpm_ensemble_advance_timestep(e, vx, vzeta, vvel, fx, fzeta, fvel, farea)) return r;
  return LPM_OK;
}

}  // extern "C"

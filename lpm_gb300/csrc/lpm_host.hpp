// lpm_host.hpp -- internal declarations shared by the library's translation
// units (not part of the public C ABI, which is include/lpm_gb300.h).
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "lpm_gb300.h"

namespace lpm {

// ---- host-only helpers (mesh.cpp, ics.cpp) --------------------------------
void mesh_sizes(int kind, int level, int64_t* nv, int64_t* nf);
// fverts (optional): nfv vertex indices per face slot, counter-clockwise
void mesh_build(int kind, int level, double radius, double* vx, double* fx,
                double* farea, uint8_t* fmask, int32_t* fverts = nullptr);
int mesh_nfv(int kind);  // vertices per face of a mesh kind
void ic_eval(int kind, const double* prm, int np, int ndim, int64_t n,
             const double* x, double* zeta);
// Level-0 mesh (the seed) with its face vertex lists (nfv per face).
struct MeshSeed {
  int ndim = 3, nfv = 3;
  bool sphere = true;
  std::vector<double> vx, fx, area;
  std::vector<int> fverts;
};
void mesh_seed(int kind, double radius, MeshSeed& out);

// An error carrying an lpm status code; the C ABI turns it into a return
// code plus the thread-local message.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

}  // namespace lpm

#ifdef __CUDACC__
#include <cuda_runtime.h>

namespace lpm {

#define LPM_CUDA(call)                                                    \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess)                                                \
      throw ::lpm::Error(LPM_ERR_CUDA, std::string(#call) + ": " +        \
                                           cudaGetErrorString(e_));       \
  } while (0)

// Makes `device` current for the lifetime of the guard and then restores the
// device that was current before, so an entry point never leaves the calling
// thread on a different GPU.  status holds cudaSetDevice's result.
struct DeviceGuard {
  int prev = -1;
  cudaError_t status = cudaSuccess;
  explicit DeviceGuard(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != device) {
      status = cudaSetDevice(device);
    } else {
      prev = -1;  // already current: nothing to restore
    }
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// Strided FP64 view, same layout as lpm_view.
struct View {
  double* p;
  int64_t si;
  int64_t sc;
  __host__ __device__ double& operator()(int64_t i, int c) const {
    return p[i * si + c * sc];
  }
};
inline View to_view(lpm_view v) { return View{v.p, v.stride_i, v.stride_c}; }

// Pair-formula families (arithmetic of the FP64 path).
enum Form : int {
  FORM_BVE = 0,    // biot_savart / greens_fn, src/lpm_sphere_functions.hpp
  FORM_SPHERE = 1, // Incompressible2DKernels<SphereGeometry> (eps form)
  FORM_PLANE = 2   // Incompressible2DKernels<PlaneGeometry>
};

// Grow-only device arena owned by a context.  A fixed arena wraps memory it
// does not own and never reallocates: reserve() beyond its capacity throws.
struct Arena {
  char* base = nullptr;
  size_t cap = 0;
  size_t off = 0;
  bool fixed = false;
  void reserve(size_t bytes);
  void reset() { off = 0; }
  void* take(size_t bytes) {
    const size_t a = (off + 255) & ~size_t(255);
    if (a + bytes > cap) throw Error(LPM_ERR_ALLOC, "arena overflow");
    off = a + bytes;
    return base + a;
  }
  void release();
};

}  // namespace lpm

struct lpm_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  int precision = LPM_FP64;
  int num_sms = 0;
  int* d_err = nullptr;  // device flag: nonzero after a bounded wait gave up
  lpm::Arena arena;
  int64_t launches = 0;
  size_t max_part_bytes = 0;  // cap on chunk-partial scratch (0 = none)
  std::map<uint64_t, int> tuned;  // autotuned FP32 kernel shape per size class
  bool autotune = true;
  int forced_shape = -1;  // >= 0: FP32 kernel shape fixed by the caller
};

namespace lpm {

// Source set: face slots with vorticity, area and the divided-face mask.
struct SrcSpec {
  View x;
  const double* zeta;
  const double* area;
  const uint8_t* mask;
  int64_t nslots;
};

// One segment of targets (e.g. vertices, or face slots).
struct TgtSeg {
  View x;           // positions, rows 0..n-1
  int64_t n;
  View u;           // output velocity (u.p may be null)
  double* psi;      // output stream function (may be null)
  bool collocated;  // row i is source slot i
};

struct SumSpec {
  int ndim;       // 2 plane, 3 sphere
  int form;       // Form
  int precision;  // LPM_FP64 or LPM_FP32C
  double eps;
  bool want_u;
  bool want_psi;
  bool skip_self;  // collocated segments skip their own slot
};

// Evaluates the direct sum for up to two target segments against one source
// set, writing into the segments' outputs (asynchronous on ctx.stream).
void direct_sum(lpm_context& ctx, const SumSpec& spec, const SrcSpec& src,
                const TgtSeg* segs, int nseg);

// Source compaction: slot2src[slot] = compacted source index or -1 (masked),
// src2slot[k] = slot of source k.  Returns the source count (synchronises).
int64_t compact_sources(lpm_context& ctx, const uint8_t* mask, int64_t nslots,
                        int* slot2src, int* src2slot);

// Launch plan of the tiled N-body kernels.
struct NbodyPlan {
  int precision;
  int ndim;
  int form;
  bool wu, wp;
  int ncomp;          // partial components per target
  int64_t ntgt, ntgt_pad;
  int64_t nsrc, nsrc_pad;
  int nchunks;
  int chunk_len;
  int nchunks_max;     // bound on nchunks for any nsrc <= this plan's nsrc
  int shape = 0;       // FP32 kernel shape (index into kF32Shapes)
  bool skipc = false;  // chord stream function: drop coincident (i == j) pairs
  size_t part_bytes() const {
    return sizeof(double) * size_t(ncomp) * size_t(nchunks) * size_t(ntgt_pad);
  }
  size_t part_bytes_max() const {
    return sizeof(double) * size_t(ncomp) * size_t(nchunks_max) * size_t(ntgt_pad);
  }
};
NbodyPlan plan_nbody(lpm_context& ctx, int precision, int ndim, int form,
                     bool wu, bool wp, int64_t ntgt, int64_t nsrc);
// tgt: float4[ntgt_pad] (FP32) or double4_16a[ntgt_pad] (FP64, with tself);
// src: float4/double4_16a[nsrc_pad].  eps: kernel smoothing.
void launch_nbody(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
                  const int* tself, const void* src, double* part,
                  double eps);
// FP32 plans: times every kernel shape on the packed arrays (one warm and
// one timed launch each) and returns the fastest; synchronises.  Results are
// cached in the context by problem size class.
int tune_shape(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
               const int* tself, const void* src, double* part, double eps);
// FP32 squared-distance offset c0 (2 eps^2 on the sphere, eps^2 on the plane,
// plus the 1e-30 floor).
float f32_c0(int ndim, double eps);
double chord_c0(int ndim, double eps);
// Deterministic sum of the .w strengths of nsrc packed source records into
// *out (scratch256: 256 doubles).
void sum_strengths(lpm_context& ctx, const void* src, bool f32, int64_t nsrc,
                   double* out, double* scratch256);

// Small device utilities (direct_sum.cu).
void bve_tendency(lpm_context& ctx, double* dzeta, View u, int64_t n,
                  double dt, double Omega);
void ic2d_tendency(lpm_context& ctx, int ndim, double* dzeta, View u,
                   int64_t n, double cor);
void tangency(lpm_context& ctx, double* out, View x, View u, int64_t n);
void invariants(lpm_context& ctx, int ndim, int64_t n, const double* zeta,
                View vel, const double* area, const uint8_t* mask,
                double out[3]);
void err_norms(lpm_context& ctx, int ndim, int64_t n, View appx, View exact,
               const double* wt, const uint8_t* mask, double out[3]);
double fma_peak(lpm_context& ctx, int precision);
// One CTA whose tile wait cannot complete: it arms the tile pipeline's
// mbarrier for a copy that is never issued, gives up after `spin` polls, sets
// the context's device error flag, drains (bounded) and returns.
void wait_selftest(lpm_context& ctx, unsigned spin);
// Uniform mesh built on the device (mesh_dev.cu); device output arrays.
void mesh_build_device(lpm_context& ctx, int kind, int level, double radius, double* vx,
                       double* fx, double* farea, uint8_t* fmask);
void check_device_error(lpm_context& ctx);

}  // namespace lpm
#endif

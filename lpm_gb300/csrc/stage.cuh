// stage.cuh -- device side of the time steppers: target/partial access for
// one problem (Tg, Pk) or an ensemble (EnsTg, EnsPk), packing of the next
// evaluation's tiles, the combine of chunk partials and the fused RK4 / RK2
// stage kernels (see stepper.cu and ensemble.cu).
#pragma once

#include <cstdint>

#include "lpm_host.hpp"
#include "nbody.cuh"

namespace lpm {
// internal linkage: every translation unit that includes this header gets its
// own copy of these kernels
namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

// Device view of the stepper's targets: vertices first, then face targets
// (all face slots, or the unmasked ones with LPM_STEP_SKIP_MASKED_TARGETS).
struct Tg {
  int ndim;
  int64_t nv, T;
  __device__ bool valid(int64_t) const { return true; }
  const int* fslot;     // face target -> face slot
  const int* slot2src;  // face slot -> source index or -1
  View vx, fx, vvel, fvel;
  double *vzeta, *fzeta, *vpsi, *fpsi;
  const double* farea;
  __device__ bool face(int64_t t) const { return t >= nv; }
  __device__ int64_t slot(int64_t t) const { return fslot[t - nv]; }
  __device__ double& x(int64_t t, int c) const {
    return face(t) ? fx(slot(t), c) : vx(t, c);
  }
  __device__ double& u(int64_t t, int c) const {
    return face(t) ? fvel(slot(t), c) : vvel(t, c);
  }
  __device__ double& zeta(int64_t t) const {
    return face(t) ? fzeta[slot(t)] : vzeta[t];
  }
  __device__ double* psi(int64_t t) const {
    return face(t) ? (fpsi ? fpsi + slot(t) : nullptr) : (vpsi ? vpsi + t : nullptr);
  }
};

// Targets of an ensemble: problem-major, each problem's targets (vertices,
// then face targets) padded to a whole number of target blocks.  tix[t] is
// the global vertex index (>= 0), -(global face slot + 1), or kPadTarget.
constexpr int kPadTarget = -2147483647 - 1;
struct EnsTg {
  int ndim;
  int64_t T;
  const int* tix;
  const int* slot2src;  // global face slot -> global source index or -1
  View vx, fx, vvel, fvel;
  double *vzeta, *fzeta, *vpsi, *fpsi;
  const double* farea;
  __device__ bool valid(int64_t t) const { return tix[t] != kPadTarget; }
  __device__ bool face(int64_t t) const { return tix[t] < 0; }
  __device__ int64_t slot(int64_t t) const { return -int64_t(tix[t]) - 1; }
  __device__ double& x(int64_t t, int c) const {
    return face(t) ? fx(slot(t), c) : vx(tix[t], c);
  }
  __device__ double& u(int64_t t, int c) const {
    return face(t) ? fvel(slot(t), c) : vvel(tix[t], c);
  }
  __device__ double& zeta(int64_t t) const {
    return face(t) ? fzeta[slot(t)] : vzeta[tix[t]];
  }
  __device__ double* psi(int64_t t) const {
    return face(t) ? (fpsi ? fpsi + slot(t) : nullptr) : (vpsi ? vpsi + tix[t] : nullptr);
  }
};

// Packed tiles and partials of one problem's evaluations.
struct Pk {
  int mode;  // M_REF64, M_C32 or M_C64
  bool exact = false;  // M_REF64: term-by-term kernel (partials are u, psi)
  int form;
  bool skip_self;
  void* tgt;
  int* tself;
  void* src;
  const double* part;
  int nchunks;
  int64_t tpad;
  // chunk count of target t, and its chunk-0 component-0 partial with the
  // component stride (the chunk stride is ncomp * stride)
  __device__ int chunks(int64_t) const { return nchunks; }
  __device__ const double* pbase(int64_t t, int64_t& stride) const {
    stride = tpad;
    return part + t;
  }
};

// Packed tiles and partials of an ensemble: per-problem partial blocks.
struct EnsPk {
  int mode;
  bool exact = false;
  int form;
  bool skip_self;
  void* tgt;
  int* tself;
  void* src;
  const double* part;
  const int* tprob;      // target -> problem
  const int64_t* pbase_;  // problem -> first partial
  const int* pchunks;    // problem -> chunk count
  const int64_t* ptpad;  // problem -> padded target count
  const int64_t* ptoff;  // problem -> first target
  __device__ int chunks(int64_t t) const { return pchunks[tprob[t]]; }
  __device__ const double* pbase(int64_t t, int64_t& stride) const {
    const int p = tprob[t];
    stride = ptpad[p];
    return part + pbase_[p] + (t - ptoff[p]);
  }
};

// Positions of all targets (T x 3) and of the sources (nsrc x 3), FP64.
__global__ void k_snapshot(Tg g, const int* src2slot, int64_t nsrc, double* tx, double* sx) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < g.T) {
    for (int c = 0; c < 3; ++c) tx[3 * i + c] = g.x(i, c);
  } else if (i < g.T + nsrc) {
    const int64_t s = i - g.T;
    for (int c = 0; c < 3; ++c) sx[3 * s + c] = g.fx(src2slot[s], c);
  }
}

// Pack target t (and its source record when it is an unmasked face) at
// position p with vorticity z.
template <class TG, class PK>
__device__ void pack(const TG& g, const PK& k, int64_t t, const double* p,
                     double z) {
  int src = -1;
  double area = 0.0;
  if (g.face(t)) {
    const int64_t s = g.slot(t);
    src = g.slot2src[s];
    area = g.farea[s];
  }
  const double p2 = g.ndim == 3 ? p[2] : 0.0;
  const bool self = k.skip_self && src >= 0;
  if (k.mode == M_C32) {
    const float gw = src >= 0 ? __double2float_rn(dm(z, area)) : 0.f;
    const float4 r = make_float4(__double2float_rn(p[0]), __double2float_rn(p[1]),
                                 __double2float_rn(p2), gw);
    static_cast<float4*>(k.tgt)[t] = make_float4(r.x, r.y, r.z, self ? gw : 0.f);
    if (src >= 0) static_cast<SrcF32*>(k.src)[src] = make_src_f32(r.x, r.y, r.z, gw);
  } else if (k.mode == M_C64) {
    const double gw = src >= 0 ? dm(z, area) : 0.0;
    static_cast<double4_16a*>(k.tgt)[t] = make_double4_16a(p[0], p[1], p2, self ? gw : 0.0);
    if (src >= 0) static_cast<double4_16a*>(k.src)[src] = make_double4_16a(p[0], p[1], p2, gw);
  } else {
    static_cast<double4_16a*>(k.tgt)[t] = make_double4_16a(p[0], p[1], p2, 0.0);
    k.tself[t] = self ? src : -1;
    if (src >= 0) {
      const double gg = (k.form == FORM_BVE) ? dm(-z, area) : dm(z, area);
      static_cast<double4_16a*>(k.src)[src] = make_double4_16a(p[0], p[1], p2, gg);
    }
  }
}

// Sum of the chunk partials of target t; chord modes turn w into u (and the
// log sum into psi) with the FP64 position p at which t was evaluated.
template <int NDIM, bool WP, class PK>
__device__ void combine_t(const PK& k, int64_t t, const double* p, double c0,
                          const double* sg, double* u, double* psi) {
  constexpr int NC = NDIM + (WP ? 1 : 0);
  double a[NC];
#pragma unroll
  for (int m = 0; m < NC; ++m) a[m] = 0.0;
  int64_t st;
  const double* b = k.pbase(t, st);
  const int nch = k.chunks(t);
  for (int c = 0; c < nch; ++c) {
    const double* q = b + (int64_t)c * NC * st;
#pragma unroll
    for (int m = 0; m < NC; ++m) a[m] += q[m * st];
  }
  if (k.mode == M_REF64) {
    if (k.exact) {
      for (int m = 0; m < NDIM; ++m) u[m] = a[m];
      if (WP) *psi = a[NDIM];
    } else {
      ref64_epilogue<NDIM, true, WP>(a, p, k.form, u, psi);
    }
    return;
  }
  if (k.mode == M_C32) {
    const double gs = (double)static_cast<const float4*>(k.tgt)[t].w;
    chord_epilogue<M_C32, NDIM, true, WP>(a, p, gs, sg, c0, u, psi);
  } else {
    const double gs = static_cast<const double4_16a*>(k.tgt)[t].w;
    chord_epilogue<M_C64, NDIM, true, WP>(a, p, gs, sg, c0, u, psi);
  }
}

template <class TG, class PK>
__device__ void combine(const TG& g, const PK& k, int64_t t, const double* p,
                        bool wp, double c0, const double* sg, double* u,
                        double* psi) {
  if (g.ndim == 3) {
    if (wp)
      combine_t<3, true>(k, t, p, c0, sg, u, psi);
    else
      combine_t<3, false>(k, t, p, c0, sg, u, psi);
  } else {
    if (wp)
      combine_t<2, true>(k, t, p, c0, sg, u, psi);
    else
      combine_t<2, false>(k, t, p, c0, sg, u, psi);
  }
}

// ---------------------------------------------------------------------------
// BVE RK4
// ---------------------------------------------------------------------------
struct Rk4Buf {
  double* xs[4];  // stage increments x_s = dt*u, SoA [3][T]
  double* zs[4];  // stage vorticity increments [T]
  double* xw;     // current evaluation positions, SoA [3][T]
};

struct Rk4Par {
  double dt, Omega;
  bool fix_facevort3, reproject;
  double c0;
};

__device__ __forceinline__ double bve_tend(double uz, double dt, double Om) {
  return dm(dm(dm(-2.0, Om), uz), dt);
}

// Stage 1 increments from the entry velocities, then stage-2 work state.
template <class TG, class PK>
__global__ void k_rk4_begin(TG g, PK k, Rk4Buf b, Rk4Par P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.T || !g.valid(t)) return;
  const int64_t T = g.T;
  double p[3];
  for (int c = 0; c < 3; ++c) {
    const double x1 = dm(P.dt, g.u(t, c));
    b.xs[0][c * T + t] = x1;
    p[c] = da(g.x(t, c), dm(0.5, x1));
    b.xw[c * T + t] = p[c];
  }
  const double z1 = bve_tend(g.u(t, 2), P.dt, P.Omega);
  b.zs[0][t] = z1;
  pack(g, k, t, p, da(g.zeta(t), dm(0.5, z1)));
}

// After evaluation s (1..3): store velocity, increments of stage s+1 and the
// work state of the next evaluation; after s == 3 apply BVERK4Update.
template <class TG, class PK>
__global__ void k_rk4_stage(TG g, PK k, Rk4Buf b, Rk4Par P, int s) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.T || !g.valid(t)) return;
  const int64_t T = g.T;
  double pw[3], u[3];
  for (int c = 0; c < 3; ++c) pw[c] = b.xw[c * T + t];
  combine(g, k, t, pw, false, P.c0, (const double*)nullptr, u, (double*)nullptr);
  for (int c = 0; c < 3; ++c) {
    g.u(t, c) = u[c];
    b.xs[s][c * T + t] = dm(P.dt, u[c]);
  }
  const double zsv = bve_tend(u[2], P.dt, P.Omega);
  b.zs[s][t] = zsv;
  double p[3];
  double z;
  if (s < 3) {
    const double cf = (s == 1) ? 0.5 : 1.0;
    for (int c = 0; c < 3; ++c) {
      p[c] = da(g.x(t, c), dm(cf, b.xs[s][c * T + t]));
      b.xw[c * T + t] = p[c];
    }
    z = da(g.zeta(t), dm(cf, zsv));
  } else {
    constexpr double sixth = 1.0 / 6.0;
    constexpr double third = 1.0 / 3.0;
    for (int c = 0; c < 3; ++c) {
      const double inc = da(dm(sixth, da(b.xs[0][c * T + t], b.xs[3][c * T + t])),
                            dm(third, da(b.xs[1][c * T + t], b.xs[2][c * T + t])));
      p[c] = da(g.x(t, c), inc);
    }
    if (P.reproject) {
      const double r = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
      for (int c = 0; c < 3; ++c) p[c] = p[c] / r;
    }
    for (int c = 0; c < 3; ++c) {
      g.x(t, c) = p[c];
      b.xw[c * T + t] = p[c];
    }
    // the reference passes facevort4 for facevort3 in the face update
    const double z3 = (g.face(t) && !P.fix_facevort3) ? b.zs[3][t] : b.zs[2][t];
    const double zinc = da(dm(sixth, da(b.zs[0][t], b.zs[3][t])),
                           dm(third, da(b.zs[1][t], z3)));
    z = da(g.zeta(t), zinc);
    g.zeta(t) = z;
  }
  pack(g, k, t, p, z);
}

template <class TG, class PK>
__global__ void k_rk4_final(TG g, PK k, Rk4Buf b, Rk4Par P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.T || !g.valid(t)) return;
  const int64_t T = g.T;
  double pw[3], u[3];
  for (int c = 0; c < 3; ++c) pw[c] = b.xw[c * T + t];
  combine(g, k, t, pw, false, P.c0, (const double*)nullptr, u, (double*)nullptr);
  for (int c = 0; c < 3; ++c) g.u(t, c) = u[c];
}

// ---------------------------------------------------------------------------
// incompressible2d RK2 (Heun)
// ---------------------------------------------------------------------------
struct Rk2Buf {
  double* x1;  // SoA [ndim][T]
  double* z1;  // [T]
  double* xw;  // SoA [ndim][T]
};
struct Rk2Par {
  double dt, cor;
  double c0;
  const double* sg;  // device: sum of source strengths (FP32 sphere psi)
};

__device__ __forceinline__ double ic2d_tend(int nd, const double* u, double cor) {
  return nd == 3 ? -dm(dm(2.0, cor), u[2]) : -dm(cor, u[1]);
}

template <class TG, class PK>
__global__ void k_rk2_begin(TG g, PK k, Rk2Buf b, Rk2Par P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.T || !g.valid(t)) return;
  const int nd = g.ndim;
  const int64_t T = g.T;
  double u[3] = {0, 0, 0}, p[3] = {0, 0, 0};
  for (int c = 0; c < nd; ++c) u[c] = g.u(t, c);
  for (int c = 0; c < nd; ++c) {
    b.x1[c * T + t] = dm(P.dt, u[c]);
    p[c] = da(g.x(t, c), dm(P.dt, u[c]));
    b.xw[c * T + t] = p[c];
  }
  const double z1 = ic2d_tend(nd, u, P.cor);
  b.z1[t] = z1;
  pack(g, k, t, p, da(g.zeta(t), dm(P.dt, z1)));
}

template <class TG, class PK>
__global__ void k_rk2_mid(TG g, PK k, Rk2Buf b, Rk2Par P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.T || !g.valid(t)) return;
  const int nd = g.ndim;
  const int64_t T = g.T;
  double pw[3] = {0, 0, 0}, u[3] = {0, 0, 0}, ps = 0;
  for (int c = 0; c < nd; ++c) pw[c] = b.xw[c * T + t];
  // velocity only: the stage's stream function would be overwritten by the
  // final evaluation
  combine(g, k, t, pw, false, P.c0, P.sg, u, &ps);
  for (int c = 0; c < nd; ++c) g.u(t, c) = u[c];
  const double z2 = ic2d_tend(nd, u, P.cor);
  const double h = dm(0.5, P.dt);
  const double z = da(da(dm(h, b.z1[t]), dm(h, z2)), g.zeta(t));
  g.zeta(t) = z;
  double p[3] = {0, 0, 0};
  for (int c = 0; c < nd; ++c) {
    const double x2 = dm(P.dt, u[c]);
    p[c] = da(da(dm(0.5, b.x1[c * T + t]), dm(0.5, x2)), g.x(t, c));
    g.x(t, c) = p[c];
    b.xw[c * T + t] = p[c];
  }
  pack(g, k, t, p, z);
}

template <class TG, class PK>
__global__ void k_rk2_final(TG g, PK k, Rk2Buf b, Rk2Par P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.T || !g.valid(t)) return;
  const int nd = g.ndim;
  const int64_t T = g.T;
  double pw[3] = {0, 0, 0}, u[3] = {0, 0, 0}, ps = 0;
  for (int c = 0; c < nd; ++c) pw[c] = b.xw[c * T + t];
  combine(g, k, t, pw, true, P.c0, P.sg, u, &ps);
  for (int c = 0; c < nd; ++c) g.u(t, c) = u[c];
  if (double* pp = g.psi(t)) *pp = ps;
}

__global__ void k_zero_bytes(char* p, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0;
}

__global__ void k_face_targets(const uint8_t* mask, int64_t nf, bool skip,
                               const int* slot2src, int* fslot) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nf) return;
  if (!skip) {
    fslot[s] = int(s);
  } else {
    const int k = slot2src[s];
    if (k >= 0) fslot[k] = int(s);
  }
}

}  // namespace
}  // namespace lpm

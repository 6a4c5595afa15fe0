// direct_sum.cu -- packing, N-body launch planning, combine epilogues and the
// small O(N) device utilities behind the functor entry points.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <cstring>
#include <vector>

#include "lpm_host.hpp"
#include "nbody.cuh"

namespace lpm {

namespace {

constexpr int SCAN_BLOCK = 1024;

__global__ void k_count_unmasked(const uint8_t* mask, int64_t n, int* bcount) {
  __shared__ int warp_counts[SCAN_BLOCK / 32];
  const int64_t i = (int64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
  const int keep = (i < n && !mask[i]) ? 1 : 0;
  const unsigned b = __ballot_sync(0xffffffffu, keep);
  if ((threadIdx.x & 31) == 0) warp_counts[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < SCAN_BLOCK / 32; ++w) s += warp_counts[w];
    bcount[blockIdx.x] = s;
  }
}

// Exclusive scan of nb block counts by one block; total in out[nb].
__global__ void k_scan_counts(const int* bcount, int nb, int* boff) {
  __shared__ int carry;
  __shared__ int wsum[SCAN_BLOCK / 32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += SCAN_BLOCK) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? bcount[i] : 0;
    int x = v;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      int w = wsum[threadIdx.x];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[threadIdx.x] = w;
    }
    __syncthreads();
    const int wprefix = (threadIdx.x >= 32) ? wsum[(threadIdx.x >> 5) - 1] : 0;
    const int incl = carry + wprefix + x;
    if (i < nb) boff[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == SCAN_BLOCK - 1) carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) boff[nb] = carry;
}

__global__ void k_scatter_map(const uint8_t* mask, int64_t n, const int* boff,
                              int* slot2src, int* src2slot) {
  __shared__ int wbase[SCAN_BLOCK / 32];
  const int64_t i = (int64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
  const int keep = (i < n && !mask[i]) ? 1 : 0;
  const unsigned b = __ballot_sync(0xffffffffu, keep);
  const int lane = threadIdx.x & 31;
  if (lane == 0) wbase[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < SCAN_BLOCK / 32; ++w) {
      const int c = wbase[w];
      wbase[w] = s;
      s += c;
    }
  }
  __syncthreads();
  if (i < n) {
    if (keep) {
      const int k = boff[blockIdx.x] + wbase[threadIdx.x >> 5] +
                    __popc(b & ((1u << lane) - 1u));
      slot2src[i] = k;
      src2slot[k] = int(i);
    } else {
      slot2src[i] = -1;
    }
  }
}

// Packed sources.  Chord modes: (x, y, z, zeta*area); FP64 reference mode:
// (x, y, z, g) with g = (-zeta)*area for the BVE form, zeta*area otherwise.
template <int MODE>
__global__ void k_pack_src(const int* src2slot, int64_t nsrc, int64_t npad,
                           View x, int ndim, const double* zeta,
                           const double* area, int form, void* out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npad) return;
  double p0 = 0, p1 = 0, p2 = 0, g = 0;
  if (k < nsrc) {
    const int64_t s = src2slot[k];
    p0 = x(s, 0);
    p1 = x(s, 1);
    if (ndim == 3) p2 = x(s, 2);
    g = (form == FORM_BVE && MODE == M_REF64) ? (-zeta[s]) * area[s] : zeta[s] * area[s];
  }
  if (MODE == M_C32) {
    reinterpret_cast<SrcF32*>(out)[k] =
        make_src_f32(__double2float_rn(p0), __double2float_rn(p1),
                     __double2float_rn(p2), __double2float_rn(g));
  } else {
    reinterpret_cast<double4_16a*>(out)[k] = make_double4_16a(p0, p1, p2, g);
  }
}

// Packed targets of one segment at offset off.  Chord modes: w = g of the
// skipped self source (for the psi self-term correction), else 0.  FP64
// reference mode: tself = skipped source index or -1.
template <int MODE>
__global__ void k_pack_tgt(int64_t off, int64_t n, View x, int ndim,
                           const int* slot2src, bool skip_self,
                           const double* zeta, const double* area, void* out,
                           int* tself) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p0 = x(i, 0), p1 = x(i, 1), p2 = ndim == 3 ? x(i, 2) : 0.0;
  int self = -1;
  if (skip_self && slot2src) self = slot2src[i];
  const double gs = self >= 0 ? zeta[i] * area[i] : 0.0;
  if (MODE == M_C32) {
    reinterpret_cast<float4*>(out)[off + i] =
        make_float4(__double2float_rn(p0), __double2float_rn(p1),
                    __double2float_rn(p2), __double2float_rn(gs));
  } else if (MODE == M_C64) {
    reinterpret_cast<double4_16a*>(out)[off + i] = make_double4_16a(p0, p1, p2, gs);
  } else {
    reinterpret_cast<double4_16a*>(out)[off + i] = make_double4_16a(p0, p1, p2, 0.0);
    tself[off + i] = self;
  }
}

__global__ void k_fill_pad_tgt(int64_t from, int64_t to, bool f32, void* out,
                               int* tself) {
  const int64_t i = from + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= to) return;
  if (f32) {
    reinterpret_cast<float4*>(out)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  } else {
    reinterpret_cast<double4_16a*>(out)[i] = make_double4_16a(0, 0, 0, 0);
    tself[i] = -1;
  }
}

// Deterministic sum of the packed source strengths (two passes).
__global__ void k_sum_g_partial(const void* src, bool f32, int64_t n, double* part) {
  __shared__ double sh[256];
  double s = 0;
  for (int64_t k = (int64_t)blockIdx.x * 256 + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * 256)
    s += f32 ? (double)static_cast<const SrcF32*>(src)[k].b.z
             : static_cast<const double4_16a*>(src)[k].w;
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_sum_final(const double* part, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += part[i];
    *out = s;
  }
}

// Combine the chunk partials of one segment and write its outputs.
template <int MODE, int NDIM, bool WU, bool WP>
__global__ void k_combine(const double* __restrict__ part, int nchunks,
                          int64_t ntgt_pad, int64_t off, int64_t n, View x,
                          View u, double* psi, const void* tgt,
                          const double* sg, double c0, int form, bool exact) {
  constexpr int NC = (WU ? NDIM : 0) + (WP ? 1 : 0);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t t = off + i;
  double a[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) a[k] = 0.0;
  for (int c = 0; c < nchunks; ++c) {
    const double* p = part + (int64_t)c * NC * ntgt_pad + t;
#pragma unroll
    for (int k = 0; k < NC; ++k) a[k] += p[k * ntgt_pad];
  }
  double pos[3] = {x(i, 0), x(i, 1), NDIM == 3 ? x(i, 2) : 0.0};
  if (MODE == M_REF64) {
    double uu[3], ps = 0;
    if (exact) {
      for (int k = 0; k < NDIM; ++k) uu[k] = a[k];
      ps = a[NC - 1];
    } else {
      ref64_epilogue<NDIM, WU, WP>(a, pos, form, uu, &ps);
    }
    if (WU)
#pragma unroll
      for (int k = 0; k < NDIM; ++k) u(i, k) = uu[k];
    if (WP) psi[i] = ps;
    return;
  }
  double uu[3], ps = 0;
  const double gs = MODE == M_C32 ? (double)static_cast<const float4*>(tgt)[t].w
                                  : static_cast<const double4_16a*>(tgt)[t].w;
  chord_epilogue<MODE, NDIM, WU, WP>(a, pos, gs, sg, c0, uu, &ps);
  if (WU)
#pragma unroll
    for (int k = 0; k < NDIM; ++k) u(i, k) = uu[k];
  if (WP) psi[i] = ps;
}

template <int MODE, int NDIM, bool WU, bool WP>
void launch_combine(lpm_context& ctx, const NbodyPlan& p, const double* part,
                    int64_t off, const TgtSeg& seg, const void* tgt,
                    const double* sg, double c0) {
  const int th = 256;
  const int64_t nb = (seg.n + th - 1) / th;
  k_combine<MODE, NDIM, WU, WP><<<nb, th, 0, ctx.stream>>>(
      part, p.nchunks, p.ntgt_pad, off, seg.n, seg.x, seg.u, seg.psi, tgt, sg, c0, p.form,
      ref64_exact(p.precision));
  ctx.launches++;
}

template <int MODE, int NDIM>
void combine_dispatch(lpm_context& ctx, const NbodyPlan& p, const double* part,
                      int64_t off, const TgtSeg& seg, const void* tgt,
                      const double* sg, double c0) {
  if (p.wu && p.wp)
    launch_combine<MODE, NDIM, true, true>(ctx, p, part, off, seg, tgt, sg, c0);
  else if (p.wu)
    launch_combine<MODE, NDIM, true, false>(ctx, p, part, off, seg, tgt, sg, c0);
  else
    launch_combine<MODE, NDIM, false, true>(ctx, p, part, off, seg, tgt, sg, c0);
}

template <typename T, int NDIM, bool WU, bool WP, bool SKIPC, int R, int NT, int MINB>
void launch_chord_shape(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
                        const void* src, double* part, T c0) {
  constexpr int TILE = std::is_same<T, float>::value ? F32_TILE : F64_TILE;
  using V4 = typename Vec4<T>::type;
  using Rec = typename SrcRec<T>::type;
  dim3 grid(unsigned(p.ntgt_pad / (NT * R)), unsigned(p.nchunks));
  nbody_chord<T, NDIM, WU, WP, SKIPC, R, NT, TILE, MINB><<<grid, NT, 0, ctx.stream>>>(
      static_cast<const V4*>(tgt), static_cast<const Rec*>(src), p.ntgt_pad, p.nsrc_pad,
      p.chunk_len, c0, part, ctx.d_err);
  ctx.launches++;
}

template <typename T, int NDIM, bool WU, bool WP, bool SKIPC>
void launch_chord_k(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
                    const void* src, double* part, T c0) {
  if constexpr (std::is_same<T, float>::value) {
    static_assert(kF32Shapes[0].nt == 256 && kF32Shapes[0].r == 4 && kF32Shapes[0].minb == 3 &&
                      kF32Shapes[1].nt == 256 && kF32Shapes[1].r == 4 && kF32Shapes[1].minb == 4 &&
                      kF32Shapes[2].nt == 128 && kF32Shapes[2].r == 8 && kF32Shapes[2].minb == 4 &&
                      kF32Shapes[3].nt == 256 && kF32Shapes[3].r == 2 && kF32Shapes[3].minb == 5 &&
                      kF32Shapes[4].nt == 128 && kF32Shapes[4].r == 8 && kF32Shapes[4].minb == 3 &&
                      kF32Shapes[5].nt == 256 && kF32Shapes[5].r == 4 && kF32Shapes[5].minb == 2 &&
                      kNumF32Shapes == 6,
                  "launch table out of sync with kF32Shapes");
    switch (p.shape) {
      case 1:
        launch_chord_shape<T, NDIM, WU, WP, SKIPC, 4, 256, 4>(ctx, p, tgt, src, part, c0);
        break;
      case 2:
        launch_chord_shape<T, NDIM, WU, WP, SKIPC, 8, 128, 4>(ctx, p, tgt, src, part, c0);
        break;
      case 3:
        launch_chord_shape<T, NDIM, WU, WP, SKIPC, 2, 256, 5>(ctx, p, tgt, src, part, c0);
        break;
      case 4:
        launch_chord_shape<T, NDIM, WU, WP, SKIPC, 8, 128, 3>(ctx, p, tgt, src, part, c0);
        break;
      case 5:
        launch_chord_shape<T, NDIM, WU, WP, SKIPC, 4, 256, 2>(ctx, p, tgt, src, part, c0);
        break;
      default:
        launch_chord_shape<T, NDIM, WU, WP, SKIPC, 4, 256, 3>(ctx, p, tgt, src, part, c0);
    }
  } else {
    launch_chord_shape<T, NDIM, WU, WP, SKIPC, F64_R, F64_NT, 4>(ctx, p, tgt, src, part, c0);
  }
}

template <typename T, int NDIM, bool WU, bool WP>
void launch_chord(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
                  const void* src, double* part, T c0) {
  if (WP && p.skipc)
    launch_chord_k<T, NDIM, WU, WP, WP>(ctx, p, tgt, src, part, c0);
  else
    launch_chord_k<T, NDIM, WU, WP, false>(ctx, p, tgt, src, part, c0);
}

template <int FORM, bool WU, bool WP>
void launch_f64(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
                const int* tself, const void* src, double* part, double eps2) {
  dim3 grid(unsigned(p.ntgt_pad / (F64_NT * F64_R)), unsigned(p.nchunks));
  if (ref64_exact(p.precision))
    nbody_f64<FORM, WU, WP, F64_R, F64_NT, F64_TILE><<<grid, F64_NT, 0, ctx.stream>>>(
        static_cast<const double4_16a*>(tgt), tself, static_cast<const double4_16a*>(src),
        p.ntgt_pad, p.nsrc_pad, p.chunk_len, eps2, part, ctx.d_err);
  else
    nbody_f64h<FORM, WU, WP, F64_R, F64_NT, F64_TILE><<<grid, F64_NT, 0, ctx.stream>>>(
        static_cast<const double4_16a*>(tgt), tself, static_cast<const double4_16a*>(src),
        p.ntgt_pad, p.nsrc_pad, p.chunk_len, eps2, part, ctx.d_err);
  ctx.launches++;
}

template <int FORM>
void f64_want(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
              const int* tself, const void* src, double* part, double eps2) {
  if (p.wu && p.wp)
    launch_f64<FORM, true, true>(ctx, p, tgt, tself, src, part, eps2);
  else if (p.wu)
    launch_f64<FORM, true, false>(ctx, p, tgt, tself, src, part, eps2);
  else
    launch_f64<FORM, false, true>(ctx, p, tgt, tself, src, part, eps2);
}

template <typename T, int NDIM>
void chord_want(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
                const void* src, double* part, T c0) {
  if (p.wu && p.wp)
    launch_chord<T, NDIM, true, true>(ctx, p, tgt, src, part, c0);
  else if (p.wu)
    launch_chord<T, NDIM, true, false>(ctx, p, tgt, src, part, c0);
  else
    launch_chord<T, NDIM, false, true>(ctx, p, tgt, src, part, c0);
}

int occupancy(int precision) {
  static int occ[3] = {0, 0, 0};
  const int m = mode_of(precision);
  int& o = occ[m];
  if (o == 0) {
    int v = 0;
    if (m == M_C32)
      v = 4;  // FP32 shapes share a fixed chunking (plan_nbody)
    else if (m == M_C64)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &v, nbody_chord<double, 3, true, false, false, F64_R, F64_NT, F64_TILE, 4>, F64_NT, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &v, nbody_f64h<0, true, false, F64_R, F64_NT, F64_TILE>, F64_NT, 0);
    o = v > 0 ? v : 1;
  }
  return o;
}

}  // namespace

float f32_c0(int ndim, double eps) { return float(chord_c0(ndim, eps)); }

double chord_c0(int ndim, double eps) {
  const double e2 = eps * eps;
  return (ndim == 3 ? 2.0 * e2 : e2) + 1e-30;
}

int64_t compact_sources(lpm_context& ctx, const uint8_t* mask, int64_t nslots,
                        int* slot2src, int* src2slot) {
  if (nslots == 0) return 0;
  const int nb = int((nslots + SCAN_BLOCK - 1) / SCAN_BLOCK);
  int* tmp = static_cast<int*>(ctx.arena.take(sizeof(int) * (2 * size_t(nb) + 1)));
  int* bcount = tmp;
  int* boff = tmp + nb;
  k_count_unmasked<<<nb, SCAN_BLOCK, 0, ctx.stream>>>(mask, nslots, bcount);
  k_scan_counts<<<1, SCAN_BLOCK, 0, ctx.stream>>>(bcount, nb, boff);
  k_scatter_map<<<nb, SCAN_BLOCK, 0, ctx.stream>>>(mask, nslots, boff, slot2src,
                                                   src2slot);
  ctx.launches += 3;
  LPM_CUDA(cudaGetLastError());
  int total = 0;
  LPM_CUDA(cudaMemcpyAsync(&total, boff + nb, sizeof(int), cudaMemcpyDeviceToHost,
                           ctx.stream));
  LPM_CUDA(cudaStreamSynchronize(ctx.stream));
  return total;
}

NbodyPlan plan_nbody(lpm_context& ctx, int precision, int ndim, int form,
                     bool wu, bool wp, int64_t ntgt, int64_t nsrc) {
  NbodyPlan p{};
  p.precision = precision;
  p.ndim = ndim;
  p.form = form;
  p.wu = wu;
  p.wp = wp;
  p.ncomp = (wu ? ndim : 0) + (wp ? 1 : 0);
  const bool f32 = precision == LPM_FP32C;
  const int tb = f32 ? F32_TB : F64_NT * F64_R;
  const int tile = f32 ? F32_TILE : F64_TILE;
  p.ntgt = ntgt;
  p.ntgt_pad = std::max<int64_t>(tb, (ntgt + tb - 1) / tb * tb);
  p.nsrc = nsrc;
  p.nsrc_pad = std::max<int64_t>(tile, (nsrc + tile - 1) / tile * tile);
  const int64_t ntb = p.ntgt_pad / tb;
  const int64_t ntiles = p.nsrc_pad / tile;
  // Aim for ~16 waves of CTAs so the tail of the last wave stays small.  The
  // FP32 shapes share one chunking (4 CTAs of 1024 targets per SM) so that the
  // autotuner can swap shapes without changing the partial layout.
  const int64_t slots = int64_t(std::max(ctx.num_sms, 1)) * (f32 ? 4 : occupancy(precision));
  int64_t nch = (16 * slots + ntb - 1) / ntb;
  if (ctx.max_part_bytes > 0) {
    const int64_t per_chunk = int64_t(sizeof(double)) * p.ncomp * p.ntgt_pad;
    nch = std::min<int64_t>(nch, int64_t(ctx.max_part_bytes) / per_chunk);
  }
  nch = std::max<int64_t>(1, std::min<int64_t>(nch, ntiles));
  // fewer sources never give more chunks than this (the rounding below can
  // raise nchunks when ntiles shrinks, but never above nch)
  p.nchunks_max = int(nch);
  const int64_t tiles_per_chunk = (ntiles + nch - 1) / nch;
  p.chunk_len = int(tiles_per_chunk * tile);
  p.nchunks = int((ntiles + tiles_per_chunk - 1) / tiles_per_chunk);
  return p;
}

void launch_nbody(lpm_context& ctx, const NbodyPlan& p, const void* tgt,
                  const int* tself, const void* src, double* part,
                  double eps) {
  const int m = mode_of(p.precision);
  if (m == M_C32) {
    const float c0 = f32_c0(p.ndim, eps);
    if (p.ndim == 3)
      chord_want<float, 3>(ctx, p, tgt, src, part, c0);
    else
      chord_want<float, 2>(ctx, p, tgt, src, part, c0);
  } else if (m == M_C64) {
    const double c0 = chord_c0(p.ndim, eps);
    if (p.ndim == 3)
      chord_want<double, 3>(ctx, p, tgt, src, part, c0);
    else
      chord_want<double, 2>(ctx, p, tgt, src, part, c0);
  } else {
    const double eps2 = eps * eps;
    if (p.form == FORM_BVE)
      f64_want<0>(ctx, p, tgt, tself, src, part, eps2);
    else if (p.form == FORM_SPHERE)
      f64_want<1>(ctx, p, tgt, tself, src, part, eps2);
    else
      f64_want<2>(ctx, p, tgt, tself, src, part, eps2);
  }
  LPM_CUDA(cudaGetLastError());
}

int tune_shape(lpm_context& ctx, const NbodyPlan& p0, const void* tgt, const int* tself,
               const void* src, double* part, double eps) {
  if (p0.precision != LPM_FP32C) return 0;
  if (ctx.forced_shape >= 0) return ctx.forced_shape;
  auto lg = [](int64_t v) {
    int k = 0;
    while ((int64_t(1) << k) < v) ++k;
    return uint64_t(k);
  };
  const uint64_t key = (uint64_t(p0.ndim) << 60) | (uint64_t(p0.wu) << 59) |
                       (uint64_t(p0.wp) << 58) | (uint64_t(p0.skipc) << 57) |
                       (lg(p0.ntgt_pad) << 8) | lg(p0.nsrc_pad);
  auto it = ctx.tuned.find(key);
  if (it != ctx.tuned.end()) return it->second;
  // below ~2e9 pairs a launch lasts a few hundred microseconds: keep the default
  if (!ctx.autotune || double(p0.ntgt_pad) * double(p0.nsrc_pad) < 2e9) {
    ctx.tuned[key] = 0;
    return 0;
  }
  cudaEvent_t e0, e1;
  LPM_CUDA(cudaEventCreate(&e0));
  LPM_CUDA(cudaEventCreate(&e1));
  int best = 0;
  float best_ms = 1e30f;
  for (int sh = 0; sh < kNumF32Shapes; ++sh) {
    NbodyPlan p = p0;
    p.shape = sh;
    launch_nbody(ctx, p, tgt, tself, src, part, eps);  // warm
    LPM_CUDA(cudaEventRecord(e0, ctx.stream));
    launch_nbody(ctx, p, tgt, tself, src, part, eps);
    LPM_CUDA(cudaEventRecord(e1, ctx.stream));
    LPM_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    LPM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) {
      best_ms = ms;
      best = sh;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx.tuned[key] = best;
  return best;
}

void sum_strengths(lpm_context& ctx, const void* src, bool f32, int64_t nsrc,
                   double* out, double* scratch256) {
  k_sum_g_partial<<<256, 256, 0, ctx.stream>>>(src, f32, nsrc, scratch256);
  k_sum_final<<<1, 32, 0, ctx.stream>>>(scratch256, 256, out);
  ctx.launches += 2;
}

namespace {
template <int MODE>
void pack_and_launch(lpm_context& ctx, const SumSpec& spec, const SrcSpec& src,
                     const TgtSeg* segs, int nseg, int64_t ntgt, const NbodyPlan& p,
                     const int* slot2src, const int* src2slot, void* srcp, void* tgtp,
                     int* tself, double* part, double* sgp) {
  const int th = 256;
  const int ndim = spec.ndim;
  k_pack_src<MODE><<<(p.nsrc_pad + th - 1) / th, th, 0, ctx.stream>>>(
      src2slot, p.nsrc, p.nsrc_pad, src.x, ndim, src.zeta, src.area, spec.form, srcp);
  ctx.launches++;
  int64_t off = 0;
  for (int s = 0; s < nseg; ++s) {
    const TgtSeg& g = segs[s];
    if (g.n > 0) {
      const int* map = g.collocated ? slot2src : nullptr;
      const bool skip = g.collocated && spec.skip_self;
      k_pack_tgt<MODE><<<(g.n + th - 1) / th, th, 0, ctx.stream>>>(
          off, g.n, g.x, ndim, map, skip, src.zeta, src.area, tgtp, tself);
      ctx.launches++;
    }
    off += g.n;
  }
  if (p.ntgt_pad > ntgt) {
    k_fill_pad_tgt<<<(p.ntgt_pad - ntgt + th - 1) / th, th, 0, ctx.stream>>>(
        ntgt, p.ntgt_pad, MODE == M_C32, tgtp, tself);
    ctx.launches++;
  }
  if (MODE != M_REF64 && spec.want_psi && ndim == 3)
    sum_strengths(ctx, srcp, MODE == M_C32, p.nsrc, sgp, sgp + 8);
  LPM_CUDA(cudaGetLastError());

  NbodyPlan pt = p;
  pt.shape = tune_shape(ctx, p, tgtp, tself, srcp, part, spec.eps);
  launch_nbody(ctx, pt, tgtp, tself, srcp, part, spec.eps);

  const double c0 = MODE == M_C32 ? double(f32_c0(ndim, spec.eps)) : chord_c0(ndim, spec.eps);
  off = 0;
  for (int s = 0; s < nseg; ++s) {
    const TgtSeg& g = segs[s];
    if (g.n > 0) {
      if (ndim == 3)
        combine_dispatch<MODE, 3>(ctx, p, part, off, g, tgtp, sgp, c0);
      else
        combine_dispatch<MODE, 2>(ctx, p, part, off, g, tgtp, sgp, c0);
    }
    off += g.n;
  }
  LPM_CUDA(cudaGetLastError());
}
}  // namespace

void direct_sum(lpm_context& ctx, const SumSpec& spec, const SrcSpec& src,
                const TgtSeg* segs, int nseg) {
  int64_t ntgt = 0;
  for (int s = 0; s < nseg; ++s) ntgt += segs[s].n;
  if (ntgt == 0) return;
  const int m = mode_of(spec.precision);
  const int ndim = spec.ndim;

  ctx.arena.reset();
  // Upper bounds first, so one reservation covers the whole call.
  NbodyPlan p = plan_nbody(ctx, spec.precision, ndim, spec.form, spec.want_u,
                           spec.want_psi, ntgt, src.nslots);
  const size_t rec = m == M_C32 ? sizeof(float4) : sizeof(double4_16a);  // target record
  const size_t srec = 32;  // source record: SrcF32 or double4_16a
  const size_t need = 4096 + sizeof(int) * (2 * size_t(src.nslots) + 2 * (size_t(src.nslots) / SCAN_BLOCK + 2)) +
                      srec * size_t(p.nsrc_pad) + rec * size_t(p.ntgt_pad) +
                      sizeof(int) * size_t(p.ntgt_pad) + p.part_bytes_max() +
                      sizeof(double) * 300 + 8 * 256;
  ctx.arena.reserve(need);

  int* slot2src = static_cast<int*>(ctx.arena.take(sizeof(int) * std::max<int64_t>(1, src.nslots)));
  int* src2slot = static_cast<int*>(ctx.arena.take(sizeof(int) * std::max<int64_t>(1, src.nslots)));
  const int64_t nsrc = compact_sources(ctx, src.mask, src.nslots, slot2src, src2slot);
  p = plan_nbody(ctx, spec.precision, ndim, spec.form, spec.want_u,
                 spec.want_psi, ntgt, nsrc);
  for (int s = 0; s < nseg; ++s)
    if (segs[s].collocated && spec.skip_self) p.skipc = true;

  void* srcp = ctx.arena.take(srec * size_t(p.nsrc_pad));
  void* tgtp = ctx.arena.take(rec * size_t(p.ntgt_pad));
  int* tself = static_cast<int*>(ctx.arena.take(sizeof(int) * size_t(p.ntgt_pad)));
  double* part = static_cast<double*>(ctx.arena.take(p.part_bytes()));
  double* sgp = static_cast<double*>(ctx.arena.take(sizeof(double) * 264));
  if (m == M_C32)
    pack_and_launch<M_C32>(ctx, spec, src, segs, nseg, ntgt, p, slot2src, src2slot, srcp,
                           tgtp, tself, part, sgp);
  else if (m == M_C64)
    pack_and_launch<M_C64>(ctx, spec, src, segs, nseg, ntgt, p, slot2src, src2slot, srcp,
                           tgtp, tself, part, sgp);
  else
    pack_and_launch<M_REF64>(ctx, spec, src, segs, nseg, ntgt, p, slot2src, src2slot, srcp,
                             tgtp, tself, part, sgp);
}

// ---------------------------------------------------------------------------
// O(N) utilities
// ---------------------------------------------------------------------------
namespace {

__global__ void k_bve_tendency(double* dz, View u, int64_t n, double dt,
                               double Omega) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dz[i] = __dmul_rn(__dmul_rn(__dmul_rn(-2.0, Omega), u(i, 2)), dt);
}

__global__ void k_tangency(double* out, View x, View u, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = __dadd_rn(__dadd_rn(__dmul_rn(x(i, 0), u(i, 0)), __dmul_rn(x(i, 1), u(i, 1))),
                       __dmul_rn(x(i, 2), u(i, 2)));
}

__global__ void k_ic2d_tendency(double* dz, View u, int64_t n, int ndim,
                                double cor) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (ndim == 3)
    dz[i] = -__dmul_rn(__dmul_rn(2.0, cor), u(i, 2));
  else
    dz[i] = -__dmul_rn(cor, u(i, 1));
}

constexpr int RED_BLOCKS = 512;
constexpr int RED_THREADS = 256;

// Block-level deterministic reduction of NV values (sum or max per slot).
template <int NV>
__device__ void block_reduce(double (&v)[NV], const bool (&is_max)[NV],
                             double* out) {
  __shared__ double sh[NV][RED_THREADS];
#pragma unroll
  for (int k = 0; k < NV; ++k) sh[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        const double a = sh[k][threadIdx.x], b = sh[k][threadIdx.x + o];
        sh[k][threadIdx.x] = is_max[k] ? fmax(a, b) : a + b;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = sh[k][0];
}

__global__ void k_invariants(int ndim, int64_t n, const double* zeta, View vel,
                             const double* area, const uint8_t* mask,
                             double* part) {
  double v[3] = {0, 0, 0};
  const bool mx[3] = {false, false, false};
  for (int64_t i = (int64_t)blockIdx.x * RED_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * RED_THREADS) {
    if (mask[i]) continue;
    const double a = area[i];
    v[0] += zeta[i] * a;
    v[1] += (zeta[i] * zeta[i]) * a;
    double n2 = 0;
    for (int k = 0; k < ndim; ++k) n2 += vel(i, k) * vel(i, k);
    v[2] += n2 * a;
  }
  block_reduce<3>(v, mx, part + 3 * blockIdx.x);
}

__global__ void k_err(int ndim, int64_t n, View appx, View exact,
                      const double* wt, const uint8_t* mask, double* part) {
  double v[6] = {0, 0, 0, 0, 0, 0};
  const bool mx[6] = {false, false, false, false, true, true};
  for (int64_t i = (int64_t)blockIdx.x * RED_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * RED_THREADS) {
    if (mask && mask[i]) continue;
    double e2 = 0, x2 = 0;
    for (int k = 0; k < ndim; ++k) {
      const double e = appx(i, k) - exact(i, k);
      e2 += e * e;
      x2 += exact(i, k) * exact(i, k);
    }
    const double em = sqrt(e2), xm = sqrt(x2), w = wt ? wt[i] : 1.0;
    v[0] += em * w;
    v[1] += xm * w;
    v[2] += em * em * w;
    v[3] += xm * xm * w;
    v[4] = fmax(v[4], em);
    v[5] = fmax(v[5], xm);
  }
  block_reduce<6>(v, mx, part + 6 * blockIdx.x);
}

template <int NV>
void finish_reduce(lpm_context& ctx, const double* dpart, double* out,
                   const bool (&is_max)[NV]) {
  std::vector<double> h(size_t(NV) * RED_BLOCKS);
  LPM_CUDA(cudaMemcpyAsync(h.data(), dpart, sizeof(double) * h.size(),
                           cudaMemcpyDeviceToHost, ctx.stream));
  LPM_CUDA(cudaStreamSynchronize(ctx.stream));
  for (int k = 0; k < NV; ++k) out[k] = 0;
  for (int b = 0; b < RED_BLOCKS; ++b)
    for (int k = 0; k < NV; ++k)
      out[k] = is_max[k] ? std::max(out[k], h[NV * b + k]) : out[k] + h[NV * b + k];
}

template <typename T>
__global__ void k_fma_peak(T* sink, int iters, T seed) {
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + T(threadIdx.x + k);
  const T b = T(0.999999), c = T(1e-7);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == T(-12345.678)) sink[threadIdx.x] = s;
}

}  // namespace

void bve_tendency(lpm_context& ctx, double* dzeta, View u, int64_t n,
                  double dt, double Omega) {
  if (n == 0) return;
  k_bve_tendency<<<(n + 255) / 256, 256, 0, ctx.stream>>>(dzeta, u, n, dt, Omega);
  ctx.launches++;
  LPM_CUDA(cudaGetLastError());
}

void tangency(lpm_context& ctx, double* out, View x, View u, int64_t n) {
  if (n == 0) return;
  k_tangency<<<(n + 255) / 256, 256, 0, ctx.stream>>>(out, x, u, n);
  ctx.launches++;
  LPM_CUDA(cudaGetLastError());
}

void ic2d_tendency(lpm_context& ctx, int ndim, double* dzeta, View u,
                   int64_t n, double cor) {
  if (n == 0) return;
  k_ic2d_tendency<<<(n + 255) / 256, 256, 0, ctx.stream>>>(dzeta, u, n, ndim, cor);
  ctx.launches++;
  LPM_CUDA(cudaGetLastError());
}

void invariants(lpm_context& ctx, int ndim, int64_t n, const double* zeta,
                View vel, const double* area, const uint8_t* mask,
                double out[3]) {
  ctx.arena.reset();
  ctx.arena.reserve(sizeof(double) * 6 * RED_BLOCKS + 256);
  double* part = static_cast<double*>(ctx.arena.take(sizeof(double) * 3 * RED_BLOCKS));
  k_invariants<<<RED_BLOCKS, RED_THREADS, 0, ctx.stream>>>(ndim, n, zeta, vel, area,
                                                           mask, part);
  ctx.launches++;
  LPM_CUDA(cudaGetLastError());
  const bool mx[3] = {false, false, false};
  finish_reduce<3>(ctx, part, out, mx);
  out[1] *= 0.5;
  out[2] *= 0.5;
}

void err_norms(lpm_context& ctx, int ndim, int64_t n, View appx, View exact,
               const double* wt, const uint8_t* mask, double out[3]) {
  ctx.arena.reset();
  ctx.arena.reserve(sizeof(double) * 6 * RED_BLOCKS + 256);
  double* part = static_cast<double*>(ctx.arena.take(sizeof(double) * 6 * RED_BLOCKS));
  k_err<<<RED_BLOCKS, RED_THREADS, 0, ctx.stream>>>(ndim, n, appx, exact, wt, mask,
                                                    part);
  ctx.launches++;
  LPM_CUDA(cudaGetLastError());
  double r[6];
  const bool mx[6] = {false, false, false, false, true, true};
  finish_reduce<6>(ctx, part, r, mx);
  const double tol = 2.220446049250313e-16;
  auto safe = [tol](double x) { return x / (x * x + tol * tol); };
  out[0] = r[0] * safe(r[1]);
  out[1] = std::sqrt(r[2] * safe(r[3]));
  out[2] = r[4] * safe(r[5]);
}

namespace {
// The failure path of every N-body kernel (TilePipe::acquire giving up, then
// TilePipe::drain): thread 0 announces a tile whose bytes never arrive, the
// bounded wait runs out, the CTA flags the error and leaves.  No global
// memory is read; the pipe's source pointer is never dereferenced.
__global__ void k_wait_selftest(unsigned spin, int* err) {
  constexpr int TILE = 16;
  __shared__ __align__(128) double4_16a sbuf[2 * TILE];
  __shared__ __align__(8) uint64_t sbar[2];
  TilePipe<double4_16a, TILE> pipe{sbuf, sbar, nullptr, 1};
  pipe.spin = spin;
  pipe.init();
  if (threadIdx.x == 0) mbar_expect_tx(&sbar[0], TILE * sizeof(double4_16a));
  if (!pipe.acquire(0)) {
    pipe.drain(0, err);
    return;
  }
  pipe.release(0);
}
}  // namespace

void wait_selftest(lpm_context& ctx, unsigned spin) {
  k_wait_selftest<<<1, 32, 0, ctx.stream>>>(spin, ctx.d_err);
  ctx.launches++;
  LPM_CUDA(cudaGetLastError());
}

double fma_peak(lpm_context& ctx, int precision) {
  const int blocks = ctx.num_sms * 8, threads = 256;
  const int iters = precision == LPM_FP32C ? 4096 : 256;
  ctx.arena.reset();
  ctx.arena.reserve(4096);
  void* sink = ctx.arena.take(threads * 8);
  cudaEvent_t e0, e1;
  LPM_CUDA(cudaEventCreate(&e0));
  LPM_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    LPM_CUDA(cudaEventRecord(e0, ctx.stream));
    if (precision == LPM_FP32C)
      k_fma_peak<float><<<blocks, threads, 0, ctx.stream>>>(static_cast<float*>(sink), iters, 1.f);
    else
      k_fma_peak<double><<<blocks, threads, 0, ctx.stream>>>(static_cast<double*>(sink), iters, 1.0);
    ctx.launches++;
    LPM_CUDA(cudaEventRecord(e1, ctx.stream));
    LPM_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    LPM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0) best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8 * 16 * double(iters) * blocks * threads;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace lpm

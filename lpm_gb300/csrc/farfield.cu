// farfield.cu -- octree evaluation of the BVE sphere velocity sum.
//
// Per evaluation (all on the context stream, capturable in a CUDA graph):
//   k_ff_sort_src   packed double4_16a sources -> Morton-ordered float4
//   k_ff_cells      per cell: centre, radius, frame, moments to order 4
//                   (FP32 per 32-point batch, FP64 across batches and threads)
//   k_ff_tblocks    per block of 128 Morton-ordered targets: centre, radius
//   k_ff_lists      per target block: tree walk with the opening criterion
//                   h <= theta (D - r_b): far cells (of >= kExactMax points;
//                   smaller accepted cells are leaves and join the near
//                   list), near leaves, and the far cells close enough
//                   (h / (D - r_b) >= rho_min) for the learned correction; a
//                   block whose lists overflow is marked for the direct sum
//   k_ff_eval       per target block: exact FP32 chord sum over the near
//                   leaves (per-leaf partials merged by TwoSum) + order-4
//                   expansion of the far cells, or the full direct sum for
//                   a marked block; writes FP64 w
//   k_ff_mlp        (mlp.cu) learned correction on tensor cores, adds to w
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include <cuda_runtime.h>

#include "farfield_dev.cuh"
#include "ffmath.cuh"
#include "nbody.cuh"

namespace lpm {

namespace {

__constant__ ff::CplxTable kCplx = ff::make_cplx_table();

__global__ void k_ff_sort_src(const double4_16a* __restrict__ src, const int* __restrict__ perm,
                              int64_t n, float4* __restrict__ ys) {
  const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  const double4_16a s = src[perm[k]];
  ys[k] = make_float4(float(s.x), float(s.y), float(s.z), float(s.w));
}

// Fixed-order block reduction of NV values held by each of 128 threads (the
// result in every thread).
template <int NV, class T>
__device__ void block_sum128(T* v, T* sh) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    T x = v[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w * NV + i] = x;
  }
  __syncthreads();
  if (t < NV) sh[4 * NV + t] = ((sh[t] + sh[NV + t]) + (sh[2 * NV + t] + sh[3 * NV + t]));
  __syncthreads();
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = sh[4 * NV + i];
  __syncthreads();
}

template <class T>
__device__ T block_max128(T x, T* sh) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_down_sync(0xffffffffu, x, o));
  if (lane == 0) sh[w] = x;
  __syncthreads();
  x = max(max(sh[0], sh[1]), max(sh[2], sh[3]));
  __syncthreads();
  return x;
}

// One CTA (128 threads) per cell.
__global__ void __launch_bounds__(128) k_ff_cells(const float4* __restrict__ ys,
                                                  const int4* __restrict__ cells, int ncells,
                                                  float theta, float rmax,
                                                  float* __restrict__ cd) {
  // FP32 throughout the per-point passes and reductions (the FP64 pipe is
  // 1/64 of FP32 on this part; the expansion is evaluated in FP32 anyway)
  __shared__ float sh[5 * 40];
  __shared__ float msh[35];
  const int cell = blockIdx.x;
  if (cell >= ncells) return;
  const int4 ci = cells[cell];
  const int s0 = ci.x, n = ci.y, t = threadIdx.x;
  // pass 1: centre, S, sum g
  float a[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int i = t; i < n; i += 128) {
    const float4 p = ys[s0 + i];
    a[0] += p.x;
    a[1] += p.y;
    a[2] += p.z;
    a[3] += fabsf(p.w);
    a[4] += p.w;
  }
  block_sum128<5>(a, sh);
  // centre and frame: one thread (FP64 is 1/64 of FP32 on this part), shared
  __shared__ float geo[16];
  __shared__ double cnorm;
  if (t == 0) {
    const double c[3] = {a[0] / n, a[1] / n, a[2] / n};
    const double cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    double nn[3] = {1, 0, 0};
    if (cn > 0) nn[0] = c[0] / cn, nn[1] = c[1] / cn, nn[2] = c[2] / cn;
    const double r[3] = {fabs(nn[2]) < 0.9 ? 0.0 : 1.0, 0.0, fabs(nn[2]) < 0.9 ? 1.0 : 0.0};
    double e1[3] = {r[1] * nn[2] - r[2] * nn[1], r[2] * nn[0] - r[0] * nn[2], r[0] * nn[1] - r[1] * nn[0]};
    const double l = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    e1[0] /= l, e1[1] /= l, e1[2] /= l;
    const double e2[3] = {nn[1] * e1[2] - nn[2] * e1[1], nn[2] * e1[0] - nn[0] * e1[2],
                          nn[0] * e1[1] - nn[1] * e1[0]};
    for (int k = 0; k < 3; ++k) {
      geo[k] = float(c[k]);
      geo[3 + k] = float(e1[k]);
      geo[6 + k] = float(e2[k]);
      geo[9 + k] = float(nn[k]);
    }
    cnorm = cn;
  }
  __syncthreads();
  const float cf[3] = {geo[0], geo[1], geo[2]};
  float qf[9];
  for (int k = 0; k < 9; ++k) qf[k] = geo[3 + k];
  const double cn = cnorm;
  // pass 2: radius about the (FP32) centre
  float hmax = 0.f;
  for (int i = t; i < n; i += 128) {
    const float4 p = ys[s0 + i];
    const float x0 = p.x - cf[0], x1 = p.y - cf[1], x2 = p.z - cf[2];
    hmax = fmaxf(hmax, x0 * x0 + x1 * x1 + x2 * x2);
  }
  const double h = sqrt(double(block_max128(hmax, sh)));
  // no target (all within rmax of the origin) can accept a cell whose radius
  // exceeds theta * (|c| + rmax): its moments are never used
  const bool skip = h > double(theta) * (cn + double(rmax));
  // pass 3: moments in the cell frame
  float m[35];
#pragma unroll
  for (int k = 0; k < 35; ++k) m[k] = 0.f;
  {
    for (int i = skip ? n : t; i < n; i += 128) {
      const float4 p = ys[s0 + i];
      const float x0 = p.x - cf[0], x1 = p.y - cf[1], x2 = p.z - cf[2];
      const float d0 = qf[0] * x0 + qf[1] * x1 + qf[2] * x2;
      const float d1 = qf[3] * x0 + qf[4] * x1 + qf[5] * x2;
      const float d2 = qf[6] * x0 + qf[7] * x1 + qf[8] * x2;
      float p0[5], p1[5], p2[5];
      p0[0] = p1[0] = p2[0] = 1.f;
#pragma unroll
      for (int k = 1; k <= 4; ++k) p0[k] = p0[k - 1] * d0, p1[k] = p1[k - 1] * d1, p2[k] = p2[k - 1] * d2;
      ff::sfor<35>([&](auto I) {
        constexpr int k = decltype(I)::value;
        m[k] = fmaf(p.w, p0[ff::mono_exp(k, 0)] * p1[ff::mono_exp(k, 1)] * p2[ff::mono_exp(k, 2)], m[k]);
      });
    }
  }
  block_sum128<35>(m, sh);
  if (t < 35) msh[t] = m[t];
  __syncthreads();
  const float* M = msh;
  // record: every thread holds the reduced moments; the fields are written
  // by different threads
  float* r = cd + int64_t(cell) * kCellF;
  if (t == 0) {
    r[0] = cf[0], r[1] = cf[1], r[2] = cf[2];
    r[3] = float(cn);
    r[4] = float(h);
    r[5] = float(a[3]);
    r[6] = float(a[4]);
    r[7] = float(n);
    for (int k = 0; k < 9; ++k) r[8 + k] = qf[k];
    for (int k = 63; k < kCellC; ++k) r[k] = 0.f;
    for (int k = kCellC + 35; k < kCellF; ++k) r[k] = 0.f;
  }
  if (t < 35) r[kCellM + t] = float(M[t]);
  if (t >= 35 && t < 45) {
    // traced moments sum g d^b |d|^2, |b| <= 2
    const int k = t - 35;
    double v = 0;
    ff::sfor<10>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int e0 = ff::mono_exp(i, 0), e1 = ff::mono_exp(i, 1), e2 = ff::mono_exp(i, 2);
      if (i == k)
        v = M[ff::mono_index(e0 + 2, e1, e2)] + M[ff::mono_index(e0, e1 + 2, e2)] +
            M[ff::mono_index(e0, e1, e2 + 2)];
    });
    r[kCellN1 + k] = float(v);
  }
  if (t == 45) {
    // sum g |d|^4
    r[kCellN2] = float(M[ff::mono_index(4, 0, 0)] + M[ff::mono_index(0, 4, 0)] +
                       M[ff::mono_index(0, 0, 4)] +
                       2.0 * (M[ff::mono_index(2, 2, 0)] + M[ff::mono_index(2, 0, 2)] +
                              M[ff::mono_index(0, 2, 2)]));
  }
  if (t >= 64 && t < 64 + 35) {
    // complex moments normalised by S h^(p+q+k)
    const int j = t - 64;
    const double S = a[3] > 0 ? a[3] : 1.0;
    const double hh = h > 0 ? h : 1.0;
    double v = 0;
    for (int m = 0; m < kCplx.nterm[j]; ++m) v += double(kCplx.coef[j][m]) * M[kCplx.idx[j][m]];
    double nrm = S;
    for (int e = 0; e < kCplx.deg[j]; ++e) nrm *= hh;
    r[kCellC + j] = float(v / nrm);
  }
}

// One CTA (128 threads) per target block: Morton-ordered FP32 positions and
// the block's bounding sphere.
__global__ void __launch_bounds__(128) k_ff_tblocks(const double4_16a* __restrict__ tgt,
                                                    const int* __restrict__ tslot,
                                                    float4* __restrict__ xt, float4* __restrict__ box) {
  __shared__ double sh[5 * 8];
  const int64_t b = blockIdx.x;
  const int t = threadIdx.x;
  const int64_t i = b * kTargetBlock + t;
  float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tslot[i] >= 0) {
    const double4_16a p = tgt[tslot[i]];
    x = make_float4(float(p.x), float(p.y), float(p.z), 1.f);
  }
  xt[i] = x;
  double a[4] = {x.x, x.y, x.z, x.w};
  block_sum128<4>(a, sh);
  const float c0 = float(a[0] / a[3]), c1 = float(a[1] / a[3]), c2 = float(a[2] / a[3]);
  double r = 0;
  if (x.w > 0) {
    const float e0 = x.x - c0, e1 = x.y - c1, e2 = x.z - c2;
    r = sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
  }
  r = block_max128(r, sh);
  if (t == 0) box[b] = make_float4(c0, c1, c2, float(r) * (1.f + 1e-6f) + 1e-7f);
}

// One thread per target block: depth-first walk from the root.
__global__ void k_ff_lists(const float* __restrict__ cd, const int4* __restrict__ cells,
                           const float4* __restrict__ box, int64_t nblocks, float theta,
                           float rho_min, int learn, int* __restrict__ far, int* __restrict__ near,
                           int* __restrict__ lrn, int4* __restrict__ cnt) {
  const int64_t b = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (b >= nblocks) return;
  const float4 bx = box[b];
  int stk[8 * 22];
  int sp = 0;
  stk[sp++] = 0;
  int nf = 0, nn = 0, nl = 0, over = 0;
  int* F = far + b * kFarCap;
  int* N = near + b * kNearCap;
  int* L = lrn + b * kLearnCap;
  while (sp > 0) {
    const int c = stk[--sp];
    const float* r = cd + int64_t(c) * kCellF;
    const float e0 = bx.x - r[0], e1 = bx.y - r[1], e2 = bx.z - r[2];
    const float D = sqrtf(e0 * e0 + e1 * e1 + e2 * e2) - bx.w;
    const float h = r[4];
    const int4 ci = cells[c];
    const bool accept = D > 0.f && h <= theta * D;
    if (accept && ci.y >= kExactMax) {
      if (nf < kFarCap) F[nf] = c;
      nf++;
      if (learn && h >= rho_min * D) {
        if (nl < kLearnCap) L[nl] = c;
        nl++;
      }
    } else if (ci.w == 0) {
      // a leaf that is near, or far but small enough to sum exactly
      if (nn < kNearCap) N[nn] = c;
      nn++;
    } else {
      if (sp + ci.w > 8 * 22) {
        over = 1;
        break;
      }
      for (int k = ci.w - 1; k >= 0; --k) stk[sp++] = ci.z + k;
    }
  }
  if (nf > kFarCap || nn > kNearCap || nl > kLearnCap) over = 1;
  cnt[b] = make_int4(min(nf, kFarCap), min(nn, kNearCap), min(nl, kLearnCap), over);
}

constexpr int kNearBuf = 512;
constexpr int kFarBatch = 16;

__device__ __forceinline__ void chord_acc(float x0, float x1, float x2, float4 s, float c0,
                                          float& w0, float& w1, float& w2) {
  const float d0 = x0 - s.x, d1 = x1 - s.y, d2 = x2 - s.z;
  const float q = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, c0)));
  const float r = s.w * rcp_approx(q);
  w0 = fmaf(r, d0, w0);
  w1 = fmaf(r, d1, w1);
  w2 = fmaf(r, d2, w2);
}

// One CTA (128 threads, one target each) per target block.
__global__ void __launch_bounds__(128) k_ff_eval(
    const float4* __restrict__ xt, const int* __restrict__ tslot,
    const float4* __restrict__ ys, int64_t nsrc, const float* __restrict__ cd,
    const int4* __restrict__ cells, const int* __restrict__ far, const int* __restrict__ near,
    const int4* __restrict__ cnt, float c0, double* __restrict__ wout, int64_t wstride) {
  __shared__ __align__(32) float4 buf[kNearBuf];  // read as 32-byte source pairs
  __shared__ float cell[kFarBatch][kCellF];
  __shared__ int4 lf[8];
  const int64_t b = blockIdx.x;
  const int t = threadIdx.x;
  const float4 x = xt[b * kTargetBlock + t];
  const int4 nc = cnt[b];
  float S0 = 0.f, S1 = 0.f, S2 = 0.f, C0 = 0.f, C1 = 0.f, C2 = 0.f;
  if (nc.w) {
    // lists overflowed: full direct sum (fallback)
    for (int64_t j0 = 0; j0 < nsrc; j0 += kNearBuf) {
      const int m = int(nsrc - j0 < kNearBuf ? nsrc - j0 : kNearBuf);
      __syncthreads();
      for (int i = t; i < m; i += 128) buf[i] = ys[j0 + i];
      __syncthreads();
      float w0 = 0.f, w1 = 0.f, w2 = 0.f;
      for (int i = 0; i < m; ++i) chord_acc(x.x, x.y, x.z, buf[i], c0, w0, w1, w2);
      two_sum_acc(S0, C0, w0);
      two_sum_acc(S1, C1, w1);
      two_sum_acc(S2, C2, w2);
    }
  } else {
    // near leaves, up to 8 per batch (<= 512 sources); the 8 leaf records are
    // loaded by 8 threads at once
    const int* N = near + b * kNearCap;
    for (int l0 = 0; l0 < nc.y; l0 += 8) {
      const int nl = min(8, nc.y - l0);
      __syncthreads();
      if (t < nl) lf[t] = cells[N[l0 + t]];
      __syncthreads();
      // sources staged as interleaved pairs (x0 x1 y0 y1 z0 z1 g0 g1) so that
      // one f32x2 instruction applies two sources to this thread's target
      float* pb = reinterpret_cast<float*>(buf);
      int o = 0;
      for (int k = 0; k < nl; ++k) {
        const int4 ci = lf[k];
        const int m = min(ci.y, kMaxLeaf);
        for (int i = t; i < m; i += 128) {
          const float4 v = ys[ci.x + i];
          float* e = pb + 8 * ((o + i) >> 1) + ((o + i) & 1);
          e[0] = v.x;
          e[2] = v.y;
          e[4] = v.z;
          e[6] = v.w;
        }
        o += m;
      }
      if ((o & 1) && t == 0) {  // odd count: a zero-strength partner at the origin
        float* e = pb + 8 * (o >> 1) + 1;
        e[0] = e[2] = e[4] = e[6] = 0.f;
      }
      __syncthreads();
      const u64 X2 = pk2(x.x, x.x), Y2 = pk2(x.y, x.y), Z2 = pk2(x.z, x.z), C02 = pk2(c0, c0);
      u64 W0 = 0ull, W1 = 0ull, W2 = 0ull;
      const ulonglong4_16a* pr = reinterpret_cast<const ulonglong4_16a*>(buf);
#pragma unroll 4
      for (int i = 0; i < (o + 1) >> 1; ++i) {
        const ulonglong4_16a s = pr[i];  // (x0 x1) (y0 y1) (z0 z1) (g0 g1)
        const u64 dx = sub2(X2, s.x), dy = sub2(Y2, s.y), dz = sub2(Z2, s.z);
        const u64 q = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, C02)));
        float qa, qb;
        upk2(q, qa, qb);
        const u64 w = mul2(s.w, pk2(rcp_approx(qa), rcp_approx(qb)));
        W0 = fma2(w, dx, W0);
        W1 = fma2(w, dy, W1);
        W2 = fma2(w, dz, W2);
      }
      float a0, b0, a1, b1, a2, b2;
      upk2(W0, a0, b0);
      upk2(W1, a1, b1);
      upk2(W2, a2, b2);
      two_sum_acc(S0, C0, a0 + b0);
      two_sum_acc(S1, C1, a1 + b1);
      two_sum_acc(S2, C2, a2 + b2);
      // leaves larger than kMaxLeaf (coincident points at the deepest level)
      for (int k = 0; k < nl; ++k) {
        const int4 ci = lf[k];
        if (ci.y <= kMaxLeaf) continue;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        for (int i = kMaxLeaf; i < ci.y; ++i) chord_acc(x.x, x.y, x.z, ys[ci.x + i], c0, v0, v1, v2);
        two_sum_acc(S0, C0, v0);
        two_sum_acc(S1, C1, v1);
        two_sum_acc(S2, C2, v2);
      }
    }
    // far cells: order-4 expansion, kFarBatch cells per batch
    const int* F = far + b * kFarCap;
    for (int f0 = 0; f0 < nc.x; f0 += kFarBatch) {
      const int nb = min(kFarBatch, nc.x - f0);
      __syncthreads();
      for (int i = t; i < nb * kCellF; i += 128) {
        const int k = i / kCellF, e = i - k * kCellF;
        cell[k][e] = cd[int64_t(F[f0 + k]) * kCellF + e];
      }
      __syncthreads();
      float w0 = 0.f, w1 = 0.f, w2 = 0.f;
      for (int k = 0; k < nb; ++k) {
        float d[3], W[3], G[3];
        ff::to_cell(cell[k], x.x, x.y, x.z, d);
        ff::expand4(cell[k], d[0], d[1], d[2], c0, W);
        ff::from_cell(cell[k], W, G);
        w0 -= G[0];
        w1 -= G[1];
        w2 -= G[2];
      }
      two_sum_acc(S0, C0, w0);
      two_sum_acc(S1, C1, w1);
      two_sum_acc(S2, C2, w2);
    }
  }
  const int64_t tt = tslot[b * kTargetBlock + t];
  if (tt >= 0) {
    wout[tt] = double(S0) + double(C0);
    wout[wstride + tt] = double(S1) + double(C1);
    wout[2 * wstride + tt] = double(S2) + double(C2);
  }
}

}  // namespace

FFDevice::~FFDevice() {
  for (void* p : allocs) cudaFree(p);
}
void* FFDevice::alloc(size_t bytes) {
  void* p = nullptr;
  LPM_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
  allocs.push_back(p);
  return p;
}

void ff_cells(lpm_context& ctx, const float4* ys, const int4* cells, int ncells, float* cd) {
  k_ff_cells<<<ncells, 128, 0, ctx.stream>>>(ys, cells, ncells, 1.0f, 1e30f, cd);
  ctx.launches++;
  LPM_CUDA(cudaGetLastError());
}

void ff_launch_tree(lpm_context& ctx, FFDevice& d, const void* tgt, const void* src, double* wout,
                    int64_t wstride, double c0, double theta, double rho_min, bool learn) {
  cudaStream_t st = ctx.stream;
  k_ff_sort_src<<<unsigned((d.nsrc + 255) / 256), 256, 0, st>>>(static_cast<const double4_16a*>(src),
                                                                 d.perm, d.nsrc, d.ys);
  k_ff_cells<<<d.ncells, 128, 0, st>>>(d.ys, d.cells, d.ncells, float(theta), d.rmax, d.cd);
  k_ff_tblocks<<<unsigned(d.nblocks), 128, 0, st>>>(static_cast<const double4_16a*>(tgt), d.tslot,
                                                    d.xt, d.box);
  k_ff_lists<<<unsigned((d.nblocks + 63) / 64), 64, 0, st>>>(d.cd, d.cells, d.box, d.nblocks,
                                                            float(theta), float(rho_min), learn,
                                                            d.far, d.near, d.lrn, d.cnt);
  k_ff_eval<<<unsigned(d.nblocks), 128, 0, st>>>(d.xt, d.tslot, d.ys, d.nsrc, d.cd,
                                                 d.cells, d.far, d.near, d.cnt, float(c0), wout,
                                                 wstride);
  ctx.launches += 5;
  LPM_CUDA(cudaGetLastError());
}

}  // namespace lpm

// ---------------------------------------------------------------------------
// lpm_farfield host methods
// ---------------------------------------------------------------------------
lpm_farfield::~lpm_farfield() {
  for (void* e : events) cudaEventDestroy(static_cast<cudaEvent_t>(e));
  delete d;
}

bool lpm_farfield::built() const { return d != nullptr && d->ncells > 0; }

void lpm_farfield::build(const double* src_xyz, int64_t nsrc, const double* tgt_xyz, int64_t ntgt) {
  using namespace lpm;
  TreeTopo tp = build_tree(src_xyz, nsrc, tgt_xyz, ntgt, leaf_max);
  ff_prepare_kernels();
  FFDevice* nd = new FFDevice();
  try {
    nd->nsrc = nsrc;
    nd->ntgt = ntgt;
    nd->ncells = int(tp.start.size());
    nd->nblocks = tp.nblocks;
    double r2 = 0;
    for (int64_t i = 0; i < ntgt; ++i)
      r2 = std::max(r2, tgt_xyz[3 * i] * tgt_xyz[3 * i] + tgt_xyz[3 * i + 1] * tgt_xyz[3 * i + 1] +
                            tgt_xyz[3 * i + 2] * tgt_xyz[3 * i + 2]);
    // targets move between tree builds: keep a generous margin
    nd->rmax = float(1.1 * std::sqrt(r2) + 0.1);
    nd->perm = static_cast<int*>(nd->alloc(sizeof(int) * nsrc));
    nd->tslot = static_cast<int*>(nd->alloc(sizeof(int) * kTargetBlock * size_t(std::max<int64_t>(nd->nblocks, 1))));
    nd->cells = static_cast<int4*>(nd->alloc(sizeof(int4) * nd->ncells));
    nd->ys = static_cast<float4*>(nd->alloc(sizeof(float4) * nsrc));
    nd->cd = static_cast<float*>(nd->alloc(sizeof(float) * kCellF * size_t(nd->ncells)));
    nd->xt = static_cast<float4*>(nd->alloc(sizeof(float4) * kTargetBlock * size_t(nd->nblocks)));
    nd->box = static_cast<float4*>(nd->alloc(sizeof(float4) * size_t(nd->nblocks)));
    nd->far = static_cast<int*>(nd->alloc(sizeof(int) * kFarCap * size_t(nd->nblocks)));
    nd->near = static_cast<int*>(nd->alloc(sizeof(int) * kNearCap * size_t(nd->nblocks)));
    nd->lrn = static_cast<int*>(nd->alloc(sizeof(int) * kLearnCap * size_t(nd->nblocks)));
    nd->cnt = static_cast<int4*>(nd->alloc(sizeof(int4) * size_t(nd->nblocks)));
    nd->counter = static_cast<int*>(nd->alloc(sizeof(int) * 4));
    std::vector<int4> ci(nd->ncells);
    for (int i = 0; i < nd->ncells; ++i) ci[i] = make_int4(tp.start[i], tp.count[i], tp.child0[i], tp.nchild[i]);
    cudaStream_t st = ctx->stream;
    LPM_CUDA(cudaMemcpyAsync(nd->perm, tp.perm.data(), sizeof(int) * nsrc, cudaMemcpyHostToDevice, st));
    if (nd->nblocks > 0)
      LPM_CUDA(cudaMemcpyAsync(nd->tslot, tp.tslot.data(), sizeof(int) * tp.tslot.size(),
                               cudaMemcpyHostToDevice, st));
    LPM_CUDA(cudaMemcpyAsync(nd->cells, ci.data(), sizeof(int4) * nd->ncells, cudaMemcpyHostToDevice, st));
    LPM_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    delete nd;
    throw;
  }
  delete d;
  d = nd;
}

void lpm_farfield::evaluate(const void* tgt, const void* src, double* wout, int64_t wstride,
                            double c0, double eps) {
  using namespace lpm;
  if (!built()) throw Error(LPM_ERR_STATE, "far field: tree not built");
  const bool learn = use_net && trained;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  if (timing) {
    for (auto& e : ev) {
      LPM_CUDA(cudaEventCreate(&e));
      events.push_back(e);
    }
    LPM_CUDA(cudaEventRecord(ev[0], ctx->stream));
  }
  ff_launch_tree(*ctx, *d, tgt, src, wout, wstride, c0, theta, rho_min, learn);
  if (timing) LPM_CUDA(cudaEventRecord(ev[1], ctx->stream));
  if (learn) ff_launch_mlp(*ctx, *d, *net, norm.data(), wout, wstride, eps, rho_min);
  if (timing) LPM_CUDA(cudaEventRecord(ev[2], ctx->stream));
}

void lpm_farfield::timings(double* tree_ms, double* net_ms, int64_t* evals) {
  using namespace lpm;
  LPM_CUDA(cudaStreamSynchronize(ctx->stream));
  double a = 0, b = 0;
  for (size_t i = 0; i + 2 < events.size(); i += 3) {
    float m0 = 0, m1 = 0;
    LPM_CUDA(cudaEventElapsedTime(&m0, static_cast<cudaEvent_t>(events[i]),
                                  static_cast<cudaEvent_t>(events[i + 1])));
    LPM_CUDA(cudaEventElapsedTime(&m1, static_cast<cudaEvent_t>(events[i + 1]),
                                  static_cast<cudaEvent_t>(events[i + 2])));
    a += m0;
    b += m1;
  }
  *tree_ms = a;
  *net_ms = b;
  *evals = int64_t(events.size() / 3);
  for (void* e : events) cudaEventDestroy(static_cast<cudaEvent_t>(e));
  events.clear();
}

void lpm_farfield::counts() {
  using namespace lpm;
  std::vector<int4> c(d->nblocks);
  LPM_CUDA(cudaMemcpyAsync(c.data(), d->cnt, sizeof(int4) * d->nblocks, cudaMemcpyDeviceToHost,
                           ctx->stream));
  LPM_CUDA(cudaStreamSynchronize(ctx->stream));
  last_far = last_near = last_learn = last_fallback = last_rows = 0;
  if (use_net && trained) {
    unsigned long long r = 0;
    LPM_CUDA(cudaMemcpy(&r, d->counter + 2, sizeof(r), cudaMemcpyDeviceToHost));
    last_rows = int64_t(r);
  }
  std::vector<int4> cells(d->ncells);
  LPM_CUDA(cudaMemcpy(cells.data(), d->cells, sizeof(int4) * d->ncells, cudaMemcpyDeviceToHost));
  std::vector<int> nearl(size_t(d->nblocks) * kNearCap);
  LPM_CUDA(cudaMemcpy(nearl.data(), d->near, sizeof(int) * nearl.size(), cudaMemcpyDeviceToHost));
  for (int64_t b = 0; b < d->nblocks; ++b) {
    if (c[b].w) {
      last_fallback++;
      continue;
    }
    last_far += c[b].x;
    last_learn += c[b].z;
    for (int k = 0; k < c[b].y; ++k) last_near += cells[nearl[b * kNearCap + k]].y;
  }
}

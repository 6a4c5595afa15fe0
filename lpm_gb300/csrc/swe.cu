// swe.cu -- shallow-water direct sums: planar with particle strength exchange
// (PlanarSWEVertexSums / PlanarSWEFaceSums, src/lpm_swe_kernels.hpp:626-876)
// and spherical (SphereVertexSums / SphereFaceSums, :723-940; see
// k_swe_sphere below).
//
// Pair term (planar_swe_sums_rhs_pse, :394-480): with d = x - y,
// R = |d|^2 + eps^2, rot = zeta A, pot = sigma A,
//   u, v         = (-d1 rot + d0 pot) / (2 pi R), (d0 rot + d1 pot) / (2 pi R)
//   du/dx, du/dy, dv/dx, dv/dy from pi R^2 and 2 pi R denominators,
//   lap(s)       = (s_y - s_x) A lapPSE(|y - x| / pse_eps) / pse_eps^2,
//                  lapPSE(r) = (40 (1 - r^2) + 10 r^4 - 2 r^6 / 3) e^{-r^2} / pi
//                  (pse::BivariateOrder8::laplacian, src/lpm_pse.hpp:66-72),
//   psi, phi     = -log(R) / (4 pi) times rot, pot.
// Reducer rules (:559-570): masked sources are skipped; with collocated
// targets (face sums with eps = 0) the i == j pair is skipped.
//
// FP64 in the reference's operation order with non-contracting intrinsics:
// every term equals the reference's except through exp/log, whose last bits
// may differ from the host library's.  One CTA = 128 targets x one chunk of
// the compacted sources (tiles of 256 in shared memory); FP64 partials per
// (chunk, component, target) are added in fixed order by the epilogue, which
// also forms the double dot product du/dx^2 + 2 du/dy dv/dx + dv/dy^2.
#include <algorithm>
#include <cmath>

#include <cuda_runtime.h>

#include "lpm_host.hpp"
#include "nbody.cuh"

namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu

namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dd(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ u64 add2(u64 a, u64 b) {
  u64 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

constexpr int kSweNT = 128;   // targets per CTA
constexpr int kSweTile = 256;  // sources per shared-memory tile
constexpr int kSweNC = 9;

struct SweSrc {
  double x, y, rot, pot, s, area;
  int slot, pad;
};

__global__ void k_swe_pack(View fx, const double* __restrict__ zeta, const double* __restrict__ sigma,
                           const double* __restrict__ area, const double* __restrict__ sfc,
                           const int* __restrict__ src2slot, int64_t ns, SweSrc* __restrict__ src) {
  const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= ns) return;
  const int64_t j = src2slot[k];
  SweSrc r;
  r.x = fx(j, 0);
  r.y = fx(j, 1);
  r.rot = dm(zeta[j], area[j]);
  r.pot = dm(sigma[j], area[j]);
  r.s = sfc[j];
  r.area = area[j];
  r.slot = int(j);
  r.pad = 0;
  src[k] = r;
}

__global__ void __launch_bounds__(kSweNT) k_swe_plane(View tx, const double* __restrict__ ts,
                                                      int64_t nt, const SweSrc* __restrict__ src,
                                                      int64_t ns, int64_t chunk_len, double eps,
                                                      double pse_eps, int collocated,
                                                      double* __restrict__ part, int64_t tpad) {
  __shared__ SweSrc tile[kSweTile];
  const int64_t i = blockIdx.x * int64_t(kSweNT) + threadIdx.x;
  const int64_t c = blockIdx.y;
  const int64_t j0 = c * chunk_len, j1 = ns < j0 + chunk_len ? ns : j0 + chunk_len;
  const bool valid = i < nt;
  const double x0 = valid ? tx(i, 0) : 0.0, x1 = valid ? tx(i, 1) : 0.0;
  const double si = valid ? ts[i] : 0.0;
  const double epssq = dm(eps, eps);
  const double pse2 = dm(pse_eps, pse_eps);
  const double twopi = 2 * kPI, fourpi = 4 * kPI;
  double r[kSweNC];
#pragma unroll
  for (int k = 0; k < kSweNC; ++k) r[k] = 0.0;
  for (int64_t t0 = j0; t0 < j1; t0 += kSweTile) {
    const int m = int(j1 - t0 < kSweTile ? j1 - t0 : kSweTile);
    __syncthreads();
    for (int q = threadIdx.x; q < m; q += kSweNT) tile[q] = src[t0 + q];
    __syncthreads();
    if (!valid) continue;
    for (int q = 0; q < m; ++q) {
      const SweSrc& y = tile[q];
      if (collocated && y.slot == i) continue;
      const double d0 = ds(x0, y.x), d1 = ds(x1, y.y);
      const double rsq = da(dm(d0, d0), dm(d1, d1));
      const double R = da(rsq, epssq);
      const double denom = dm(twopi, R);
      const double denom2 = dm(kPI, dm(R, R));
      const double greens = dd(-log(R), fourpi);
      const double xy = dm(d0, d1);
      const double d00 = dm(d0, d0), d11 = dm(d1, d1);
      r[0] = da(r[0], dd(da(dm(-d1, y.rot), dm(d0, y.pot)), denom));
      r[1] = da(r[1], dd(da(dm(d0, y.rot), dm(d1, y.pot)), denom));
      r[2] = da(r[2], da(dd(ds(dm(xy, y.rot), dm(d00, y.pot)), denom2), dd(y.pot, denom)));
      r[3] = da(r[3], ds(dd(ds(dm(d11, y.rot), dm(xy, y.pot)), denom2), dd(y.rot, denom)));
      r[4] = da(r[4], da(dd(ds(dm(-d00, y.rot), dm(xy, y.pot)), denom2), dd(y.rot, denom)));
      r[5] = da(r[5], da(dd(ds(dm(-xy, y.rot), dm(d11, y.pot)), denom2), dd(y.pot, denom)));
      const double e0 = ds(y.x, x0), e1 = ds(y.y, x1);
      const double pr = dd(__dsqrt_rn(da(dm(e0, e0), dm(e1, e1))), pse_eps);
      const double p2 = dm(pr, pr);
      const double p4 = dm(p2, p2);
      const double pre = ds(da(dm(40.0, ds(1.0, p2)), dm(10.0, p4)), dd(dm(dm(2.0, p2), p4), 3.0));
      const double lap = dm(pre, dd(exp(-p2), kPI));
      r[6] = da(r[6], dd(dm(dm(ds(y.s, si), y.area), lap), pse2));
      r[7] = da(r[7], dm(greens, y.rot));
      r[8] = da(r[8], dm(greens, y.pot));
    }
  }
  if (!valid) return;
#pragma unroll
  for (int k = 0; k < kSweNC; ++k) part[(c * kSweNC + k) * tpad + i] = r[k];
}

struct SweOut {
  View u;
  double *ddot, *du1dx1, *du1dx2, *du2dx1, *du2dx2, *laps, *psi, *phi;
  int do_velocity;
};

__global__ void k_swe_out(const double* __restrict__ part, int nchunks, int64_t tpad, int64_t nt,
                          SweOut o) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  double s[kSweNC];
#pragma unroll
  for (int k = 0; k < kSweNC; ++k) s[k] = 0.0;
  for (int c = 0; c < nchunks; ++c)
#pragma unroll
    for (int k = 0; k < kSweNC; ++k) s[k] = da(s[k], part[(int64_t(c) * kSweNC + k) * tpad + i]);
  if (o.do_velocity) {
    o.u(i, 0) = s[0];
    o.u(i, 1) = s[1];
  }
  // square(du/dx) + 2 du/dy dv/dx + square(dv/dy)
  o.ddot[i] = da(da(dm(s[2], s[2]), dm(dm(2.0, s[3]), s[4])), dm(s[5], s[5]));
  o.du1dx1[i] = s[2];
  o.du1dx2[i] = s[3];
  o.du2dx1[i] = s[4];
  o.du2dx2[i] = s[5];
  o.laps[i] = s[6];
  o.psi[i] = s[7];
  o.phi[i] = s[8];
}

// ---- planar SWE sums, FP32 compensated (context precision LPM_FP32C) ------
// With d = x - y, R = |d|^2 + eps^2, r = 1/R, a = rot r, b = pot r, every
// output is a sum of per-pair moments (15 per target):
//   w0..3 = sum a d0, a d1, b d0, b d1      w4, w5 = sum a, sum b
//   w6..8 = sum a r (d0^2, d0 d1, d1^2)     w9..11 = the same with b
//   w12 = sum (s_y - s_x) A lapPSE(|d|^2 / pse_eps^2)
//   w13, w14 = sum rot lg2 R, sum pot lg2 R
// and the FP64 epilogue forms u = (-w1 + w2) / 2pi, v = (w0 + w3) / 2pi,
// du/dx = (w7 - w9) / pi + w5 / 2pi, du/dy = (w8 - w10) / pi - w4 / 2pi,
// dv/dx = (-w6 - w10) / pi + w4 / 2pi, dv/dy = (-w7 - w11) / pi + w5 / 2pi,
// lap = w12 / (pi pse_eps^2), psi, phi = -(ln 2 / 4pi) w13, w14.  The PSE
// kernel uses |d|^2 directly (the reference's sqrt then square is the
// identity).  Positions and surface heights are split into FP32 hi + lo parts
// (d and s_y - s_x are small differences of O(1) values).  Three MUFU
// results (reciprocal, log2, exp2) and ~45 FP32 operations per pair, two
// sources per packed f32x2 instruction (pair k holds sources 2k, 2k + 1; an
// odd count ends with a zero-strength, zero-area source), the sums kept per
// lane over a 256-source tile and then merged by TwoSum.
constexpr int kPl32NC = 15;

struct __align__(16) PlPair32 {
  float4 hxy;  // x hi of sources 2k, 2k + 1; y hi
  float4 lxy;  // x lo; y lo
  float4 rp;   // rot; pot
  float4 as;   // area; surface hi
  float4 sl;   // surface lo; slot (int bits)
};

__global__ void k_swe_plane32_pack(View fx, const double* __restrict__ zeta,
                                   const double* __restrict__ sigma,
                                   const double* __restrict__ area, const double* __restrict__ sfc,
                                   const int* __restrict__ src2slot, int64_t ns,
                                   PlPair32* __restrict__ src) {
  const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= (ns + 1) / 2) return;
  float v[2][9] = {};
  int sl[2] = {-1, -1};
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    if (2 * k + e >= ns) break;
    const int64_t j = src2slot[2 * k + e];
    const double x = fx(j, 0), y = fx(j, 1), sv = sfc[j];
    const float xh = float(x), yh = float(y), sh = float(sv);
    v[e][0] = xh;
    v[e][1] = yh;
    v[e][2] = float(x - xh);
    v[e][3] = float(y - yh);
    v[e][4] = float(zeta[j] * area[j]);
    v[e][5] = float(sigma[j] * area[j]);
    v[e][6] = float(area[j]);
    v[e][7] = sh;
    v[e][8] = float(sv - sh);
    sl[e] = int(j);
  }
  PlPair32 r;
  r.hxy = make_float4(v[0][0], v[1][0], v[0][1], v[1][1]);
  r.lxy = make_float4(v[0][2], v[1][2], v[0][3], v[1][3]);
  r.rp = make_float4(v[0][4], v[1][4], v[0][5], v[1][5]);
  r.as = make_float4(v[0][6], v[1][6], v[0][7], v[1][7]);
  r.sl = make_float4(v[0][8], v[1][8], __int_as_float(sl[0]), __int_as_float(sl[1]));
  src[k] = r;
}

// One pair record against one target.  COLL: face targets; the source in the
// target's own slot is skipped (its reciprocal and logarithm are replaced by
// 0, and its PSE term is 0: d = 0 and s_y - s_x = 0).  TAIL: the record may
// hold the zero-strength dummy (slot -1, at the origin, which can coincide
// with a target), whose reciprocal and logarithm are zeroed the same way.
struct Pl32Target {
  u64 x0h, x1h, sh, x0l, x1l, sl, e2, ipse2;
  int64_t i;
};

template <bool COLL, bool TAIL>
__device__ __forceinline__ void pl32_pair(const PlPair32& s, const Pl32Target& t,
                                          u64 (&w)[kPl32NC]) {
  const u64 d0 = add2(sub2(t.x0h, pk2(s.hxy.x, s.hxy.y)), sub2(t.x0l, pk2(s.lxy.x, s.lxy.y)));
  const u64 d1 = add2(sub2(t.x1h, pk2(s.hxy.z, s.hxy.w)), sub2(t.x1l, pk2(s.lxy.z, s.lxy.w)));
  const u64 dd = fma2(d0, d0, mul2(d1, d1));
  float qa, qb;
  upk2(add2(dd, t.e2), qa, qb);
  float ra = rcp_approx(qa), rb = rcp_approx(qb);
  float la = lg2_approx(qa), lb = lg2_approx(qb);
  if (COLL || TAIL) {
    const int sa = __float_as_int(s.sl.z), sb = __float_as_int(s.sl.w);
    const bool ska = (COLL && sa == t.i) || (TAIL && sa < 0);
    const bool skb = (COLL && sb == t.i) || (TAIL && sb < 0);
    ra = ska ? 0.f : ra;
    la = ska ? 0.f : la;
    rb = skb ? 0.f : rb;
    lb = skb ? 0.f : lb;
  }
  const u64 r = pk2(ra, rb), L = pk2(la, lb);
  const u64 p2 = mul2(dd, t.ipse2);
  float ea, eb;
  upk2(mul2(p2, pk2(-1.4426950408889634f, -1.4426950408889634f)), ea, eb);
  float xa, xb;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(xa) : "f"(ea));
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(xb) : "f"(eb));
  const u64 poly = fma2(fma2(fma2(pk2(-2.f / 3.f, -2.f / 3.f), p2, pk2(10.f, 10.f)), p2,
                             pk2(-40.f, -40.f)),
                        p2, pk2(40.f, 40.f));
  const u64 ds = add2(sub2(pk2(s.as.z, s.as.w), t.sh), sub2(pk2(s.sl.x, s.sl.y), t.sl));
  const u64 rot = pk2(s.rp.x, s.rp.y), pot = pk2(s.rp.z, s.rp.w);
  const u64 a = mul2(rot, r), b = mul2(pot, r);
  const u64 a2 = mul2(a, r), b2 = mul2(b, r);
  w[0] = fma2(a, d0, w[0]);
  w[1] = fma2(a, d1, w[1]);
  w[2] = fma2(b, d0, w[2]);
  w[3] = fma2(b, d1, w[3]);
  w[4] = add2(w[4], a);
  w[5] = add2(w[5], b);
  const u64 ad0 = mul2(a2, d0), ad1 = mul2(a2, d1), bd0 = mul2(b2, d0), bd1 = mul2(b2, d1);
  w[6] = fma2(ad0, d0, w[6]);
  w[7] = fma2(ad0, d1, w[7]);
  w[8] = fma2(ad1, d1, w[8]);
  w[9] = fma2(bd0, d0, w[9]);
  w[10] = fma2(bd0, d1, w[10]);
  w[11] = fma2(bd1, d1, w[11]);
  w[12] = fma2(mul2(ds, pk2(s.as.x, s.as.y)), mul2(poly, pk2(xa, xb)), w[12]);
  w[13] = fma2(rot, L, w[13]);
  w[14] = fma2(pot, L, w[14]);
}

template <bool COLL>
__global__ void __launch_bounds__(kSweNT) k_swe_plane32(View tx, const double* __restrict__ ts,
                                                        int64_t nt, const PlPair32* __restrict__ src,
                                                        int64_t ns, int64_t chunk_len, float e2,
                                                        float ipse2, double* __restrict__ part,
                                                        int64_t tpad) {
  __shared__ PlPair32 tile[kSweTile / 2];
  const int64_t i = blockIdx.x * int64_t(kSweNT) + threadIdx.x;
  const int64_t c = blockIdx.y;
  const int64_t j0 = c * chunk_len, j1 = ns < j0 + chunk_len ? ns : j0 + chunk_len;
  const bool valid = i < nt;
  const double X0 = valid ? tx(i, 0) : 0.0, X1 = valid ? tx(i, 1) : 0.0;
  const double SX = valid ? ts[i] : 0.0;
  const float x0h = float(X0), x1h = float(X1), sxh = float(SX);
  const float x0l = float(X0 - x0h), x1l = float(X1 - x1h), sxl = float(SX - sxh);
  const Pl32Target t{pk2(x0h, x0h), pk2(x1h, x1h), pk2(sxh, sxh), pk2(x0l, x0l),
                     pk2(x1l, x1l), pk2(sxl, sxl), pk2(e2, e2),  pk2(ipse2, ipse2), i};
  float S[kPl32NC], C[kPl32NC];
#pragma unroll
  for (int k = 0; k < kPl32NC; ++k) S[k] = C[k] = 0.f;
  for (int64_t t0 = j0; t0 < j1; t0 += kSweTile) {  // t0 is even: chunks are whole tiles
    const int m = int(j1 - t0 < kSweTile ? j1 - t0 : kSweTile);
    const int mp = (m + 1) / 2;
    __syncthreads();
    for (int q = threadIdx.x; q < mp; q += kSweNT) tile[q] = src[t0 / 2 + q];
    __syncthreads();
    if (!valid) continue;
    u64 w[kPl32NC];
#pragma unroll
    for (int k = 0; k < kPl32NC; ++k) w[k] = 0ull;
#pragma unroll 2
    for (int q = 0; q < m / 2; ++q) pl32_pair<COLL, false>(tile[q], t, w);
    if (m & 1) pl32_pair<COLL, true>(tile[mp - 1], t, w);  // the dummy's pair
#pragma unroll
    for (int k = 0; k < kPl32NC; ++k) {
      float a, b;
      upk2(w[k], a, b);
      two_sum_acc(S[k], C[k], a);
      two_sum_acc(S[k], C[k], b);
    }
  }
  if (!valid) return;
#pragma unroll
  for (int k = 0; k < kPl32NC; ++k) part[(c * kPl32NC + k) * tpad + i] = double(S[k]) + double(C[k]);
}

__global__ void k_swe_plane32_out(const double* __restrict__ part, int nchunks, int64_t tpad,
                                  int64_t nt, double pse_eps, SweOut o) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  double w[kPl32NC];
#pragma unroll
  for (int k = 0; k < kPl32NC; ++k) w[k] = 0.0;
  for (int c = 0; c < nchunks; ++c)
#pragma unroll
    for (int k = 0; k < kPl32NC; ++k) w[k] += part[(int64_t(c) * kPl32NC + k) * tpad + i];
  const double ipi = 1.0 / kPI, i2pi = 0.5 / kPI;
  if (o.do_velocity) {
    o.u(i, 0) = (w[2] - w[1]) * i2pi;
    o.u(i, 1) = (w[0] + w[3]) * i2pi;
  }
  const double g00 = (w[7] - w[9]) * ipi + w[5] * i2pi;
  const double g01 = (w[8] - w[10]) * ipi - w[4] * i2pi;
  const double g10 = -(w[6] + w[10]) * ipi + w[4] * i2pi;
  const double g11 = -(w[7] + w[11]) * ipi + w[5] * i2pi;
  o.ddot[i] = da(da(dm(g00, g00), dm(dm(2.0, g01), g10)), dm(g11, g11));
  o.du1dx1[i] = g00;
  o.du1dx2[i] = g01;
  o.du2dx1[i] = g10;
  o.du2dx2[i] = g11;
  o.laps[i] = w[12] * ipi / (pse_eps * pse_eps);
  const double k = -0.6931471805599453 / (4 * kPI);
  o.psi[i] = k * w[13];
  o.phi[i] = k * w[14];
}

// ---- spherical SWE sums ----------------------------------------------------
// Pair term (sphere_swe_velocity_sums, :335-373) with s = x.y,
// D = (1 - s) + eps^2, c = x cross y, rot = -zeta A, pot = -sigma A, and
// P = I - x x^T:
//   u += c rot / (4 pi D) + P y pot / (4 pi D)
//   M += gkz rot + gks pot, where the reference's polynomials for grad_kzeta
//   and grad_ksigma (:114-325) equal, over 4 pi D^2 (gkz identically, gks on
//   the unit sphere),
//     gkz = D [y]x + c v^T,          v = (1 + eps^2) x - y
//     gks = -v w^T - D s P,          w = P y = y - s x
//   (w - D x = -v because s + D = 1 + eps^2).
// Per target the terms linear in [y]x and P are summed as a vector and a
// scalar and applied once:
//   M = sum_j (R c) v^T - (Q v) w^T + [sum_j rot y / (4 pi D)]x
//       - (sum_j s pot / (4 pi D)) P,      R, Q = rot, pot / (4 pi D^2).
// FP64: s and D = (1 - s) + eps^2 unfused in the reference's order (D is
// the ill-conditioned quantity: a one-ulp change of s moves a near pair's D by
// ~1e-16 / D relative), everything after it contracted, one reciprocal of D per
// pair (Newton-Raphson from an FP32 seed, two steps: relative error below
// 1e-28 before the final rounding); about 66 FP64 instructions per pair
// against ~210 for the non-contracted three-division form.  Agreement with
// the oracle (which keeps the reference's operation order) is ~1e-14
// relative.
constexpr int kSphNC = 16;  // u[3], Mr[9], Yd[3], G

struct SphSrc {
  double x, y, z, rot, pot;
  int slot, pad;
};

__global__ void k_swe_sphere_pack(View fx, const double* __restrict__ zeta,
                                  const double* __restrict__ sigma, const double* __restrict__ area,
                                  const int* __restrict__ src2slot, int64_t ns,
                                  SphSrc* __restrict__ src) {
  const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= ns) return;
  const int64_t j = src2slot[k];
  SphSrc r;
  r.x = fx(j, 0);
  r.y = fx(j, 1);
  r.z = fx(j, 2);
  r.rot = -zeta[j] * area[j];
  r.pot = -sigma[j] * area[j];
  r.slot = int(j);
  r.pad = 0;
  src[k] = r;
}

// 1/d by Newton-Raphson, r <- r + r (1 - d r), from the FP32 reciprocal.
__device__ __forceinline__ double recip_nr(double d) {
  double r = double(__frcp_rn(float(d)));
  r = fma(r, fma(-d, r, 1.0), r);
  return fma(r, fma(-d, r, 1.0), r);
}

__global__ void __launch_bounds__(kSweNT) k_swe_sphere(View tx, int64_t nt,
                                                       const SphSrc* __restrict__ src, int64_t ns,
                                                       int64_t chunk_len, double eps,
                                                       int collocated, double* __restrict__ part,
                                                       int64_t tpad) {
  __shared__ SphSrc tile[kSweTile];
  const int64_t i = blockIdx.x * int64_t(kSweNT) + threadIdx.x;
  const int64_t c = blockIdx.y;
  const int64_t j0 = c * chunk_len, j1 = ns < j0 + chunk_len ? ns : j0 + chunk_len;
  const bool valid = i < nt;
  double x[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) x[a] = valid ? tx(i, a) : 0.0;
  const double epssq = eps * eps;
  const double e1 = 1.0 + epssq;
  const double inv4pi = 1.0 / (4 * kPI);
  const double ex[3] = {e1 * x[0], e1 * x[1], e1 * x[2]};
  double r[kSphNC];
#pragma unroll
  for (int k = 0; k < kSphNC; ++k) r[k] = 0.0;
  for (int64_t t0 = j0; t0 < j1; t0 += kSweTile) {
    const int m = int(j1 - t0 < kSweTile ? j1 - t0 : kSweTile);
    __syncthreads();
    for (int q = threadIdx.x; q < m; q += kSweNT) tile[q] = src[t0 + q];
    __syncthreads();
    if (!valid) continue;
#pragma unroll 2
    for (int q = 0; q < m; ++q) {
      const SphSrc& sr = tile[q];
      if (collocated && sr.slot == i) continue;
      const double y[3] = {sr.x, sr.y, sr.z};
      // x.y unfused in the reference's order: D = 1 - s cancels, and its
      // rounding is the reference's
      const double s = da(da(dm(x[0], y[0]), dm(x[1], y[1])), dm(x[2], y[2]));
      const double D = da(ds(1.0, s), epssq);
      const double rd = recip_nr(D);
      const double inv1 = rd * inv4pi;  // 1 / (4 pi D)
      const double den2 = inv1 * rd;    // 1 / (4 pi D^2)
      const double sz = sr.rot * inv1, ss = sr.pot * inv1;
      const double R = sr.rot * den2, Q = sr.pot * den2;
      const double cr[3] = {fma(x[1], y[2], -x[2] * y[1]), fma(x[2], y[0], -x[0] * y[2]),
                            fma(x[0], y[1], -x[1] * y[0])};
      double w[3], v[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        w[a] = fma(-s, x[a], y[a]);
        v[a] = ex[a] - y[a];
        r[a] = fma(cr[a], sz, fma(w[a], ss, r[a]));
        r[12 + a] = fma(sz, y[a], r[12 + a]);
      }
      r[15] = fma(ss, s, r[15]);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double al = R * cr[a], be = Q * v[a];
#pragma unroll
        for (int b = 0; b < 3; ++b) r[3 + 3 * a + b] = fma(al, v[b], fma(-be, w[b], r[3 + 3 * a + b]));
      }
    }
  }
  if (!valid) return;
#pragma unroll
  for (int k = 0; k < kSphNC; ++k) part[(c * kSphNC + k) * tpad + i] = r[k];
}

__global__ void k_swe_sphere_out(const double* __restrict__ part, int nchunks, int64_t tpad,
                                 View tx, int64_t nt, View u, double* __restrict__ ddot,
                                 double* __restrict__ grad, int do_velocity) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  double s[kSphNC];
#pragma unroll
  for (int k = 0; k < kSphNC; ++k) s[k] = 0.0;
  for (int c = 0; c < nchunks; ++c)
#pragma unroll
    for (int k = 0; k < kSphNC; ++k) s[k] += part[(int64_t(c) * kSphNC + k) * tpad + i];
  if (do_velocity) {
    u(i, 0) = s[0];
    u(i, 1) = s[1];
    u(i, 2) = s[2];
  }
  const double x[3] = {tx(i, 0), tx(i, 1), tx(i, 2)};
  const double* Yd = s + 12;
  const double Yx[9] = {0.0, -Yd[2], Yd[1], Yd[2], 0.0, -Yd[0], -Yd[1], Yd[0], 0.0};
  double M[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const double P = (a == b ? 1.0 : 0.0) - x[a] * x[b];
      M[3 * a + b] = s[3 + 3 * a + b] + Yx[3 * a + b] - s[15] * P;
    }
  // sum_ij M_ij M_ji in the functors' loop order
  double dsum = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) dsum = da(dsum, dm(M[3 * a + b], M[3 * b + a]));
  ddot[i] = dsum;
  if (grad)
#pragma unroll
    for (int k = 0; k < 9; ++k) grad[9 * i + k] = M[k];
}

// ---- spherical SWE sums, FP32 compensated (context precision LPM_FP32C) ----
// Chord form: with d = x - y for unit vectors, 1 - x.y = |d|^2 / 2, so
// D = q / 2 with q = |d|^2 + 2 eps^2, and c = x cross y = d cross x,
// v = eps^2 x + d, w = P y = -P d.  Writing rs, ps = rot, pot / (2 pi) and
// r = 1/q, the pair scalars are sz = rs r, ss = ps r (= rot, pot / (4 pi D))
// and R = 2 sz r, Q = 2 ss r (= rot, pot / (4 pi D^2)).  Every term is then a
// moment of d, summed per target (27 sums):
//   A = sum sz d, B = sum ss d, U1 = sum R d, V1 = sum Q d,
//   U2 = sum R d d^T, V2 = sum Q d d^T (symmetric), Z = sum sz, G = sum ss,
//   H = sum ss |d|^2,
// and the epilogue (FP64) assembles
//   u = A x x - P B
//   M = eps^2 (U1 x x) x^T + [U2 columns] x x + eps^2 x (P V1)^T + V2 P
//       + [Z x - A]x - (G - H/2) P.
// Positions are split into FP32 hi + lo parts so that d = (xh - yh) +
// (xl - yl) carries its own FP32 rounding, not the positions' (near pairs
// dominate the gradient: their |d| shrinks with the mesh).  Per pair: 50 FP32
// operations and one MUFU reciprocal (the strengths are stored doubled, as
// rot, pot / pi, so that R, Q = sz r, ss r need no doubling; the epilogue
// halves the sums of sz and ss, exactly).  Two sources per packed f32x2
// instruction: pair k of the packed array holds sources 2k and 2k + 1 (an odd
// count ends with a zero-strength source at the origin, whose terms are
// exactly 0), each thread owns one target, and the 27 sums are kept per lane
// (even and odd sources) over a 256-source tile; the two lanes' tile
// partials are then added into FP64 running sums in shared memory (which
// frees the registers the packed sums need).
constexpr int kSph32NC = 27;  // A3 B3 U1[3] V1[3] U2[6] V2[6] Z G H

struct __align__(16) SphPair32 {
  float4 hxy;  // x hi of sources 2k, 2k + 1; y hi of 2k, 2k + 1
  float4 hzr;  // z hi; rot / pi (twice rs: see above)
  float4 lxy;  // x lo (x - x hi); y lo
  float4 lzp;  // z lo; pot / pi
};

__global__ void k_swe_sphere32_pack(View fx, const double* __restrict__ zeta,
                                    const double* __restrict__ sigma,
                                    const double* __restrict__ area,
                                    const int* __restrict__ src2slot, int64_t ns,
                                    SphPair32* __restrict__ src, int2* __restrict__ slot) {
  const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= (ns + 1) / 2) return;
  const double inv_pi = 1.0 / kPI;  // strengths stored doubled: rot, pot / pi
  float h[2][4] = {}, l[2][4] = {};
  int sl[2] = {-1, -1};
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    if (2 * k + e >= ns) break;
    const int64_t j = src2slot[2 * k + e];
    const double x = fx(j, 0), y = fx(j, 1), z = fx(j, 2);
    h[e][0] = float(x);
    h[e][1] = float(y);
    h[e][2] = float(z);
    h[e][3] = float(-zeta[j] * area[j] * inv_pi);
    l[e][0] = float(x - double(h[e][0]));
    l[e][1] = float(y - double(h[e][1]));
    l[e][2] = float(z - double(h[e][2]));
    l[e][3] = float(-sigma[j] * area[j] * inv_pi);
    sl[e] = int(j);
  }
  SphPair32 r;
  r.hxy = make_float4(h[0][0], h[1][0], h[0][1], h[1][1]);
  r.hzr = make_float4(h[0][2], h[1][2], h[0][3], h[1][3]);
  r.lxy = make_float4(l[0][0], l[1][0], l[0][1], l[1][1]);
  r.lzp = make_float4(l[0][2], l[1][2], l[0][3], l[1][3]);
  src[k] = r;
  slot[k] = make_int2(sl[0], sl[1]);
}

// COLL: face targets; the source in the target's own slot is skipped (its
// reciprocal is replaced by 0, which zeroes every term of the pair).
template <bool COLL>
__global__ void __launch_bounds__(kSweNT, 4) k_swe_sphere32(View tx, int64_t nt,
                                                            const SphPair32* __restrict__ src,
                                                            const int2* __restrict__ slot,
                                                            int64_t ns, int64_t chunk_len, float c0,
                                                            double* __restrict__ part,
                                                            int64_t tpad) {
  __shared__ SphPair32 tile[kSweTile / 2];
  __shared__ int2 tslot[COLL ? kSweTile / 2 : 1];
  __shared__ double acc[kSph32NC][kSweNT];
  const int tid = threadIdx.x;
  const int64_t i = blockIdx.x * int64_t(kSweNT) + tid;
  const int64_t c = blockIdx.y;
  const int64_t j0 = c * chunk_len, j1 = ns < j0 + chunk_len ? ns : j0 + chunk_len;
  const bool valid = i < nt;
  u64 XH[3], XL[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double v = valid ? tx(i, a) : 0.0;
    const float h = float(v), l = float(v - double(h));
    XH[a] = pk2(h, h);
    XL[a] = pk2(l, l);
  }
  const u64 C02 = pk2(c0, c0);
#pragma unroll
  for (int k = 0; k < kSph32NC; ++k) acc[k][tid] = 0.0;
  for (int64_t t0 = j0; t0 < j1; t0 += kSweTile) {  // t0 is even: chunks are whole tiles
    const int m = int(j1 - t0 < kSweTile ? j1 - t0 : kSweTile);
    const int mp = (m + 1) / 2;
    __syncthreads();
    for (int q = tid; q < mp; q += kSweNT) {
      tile[q] = src[t0 / 2 + q];
      if (COLL) tslot[q] = slot[t0 / 2 + q];
    }
    __syncthreads();
    if (!valid) continue;
    u64 w[kSph32NC];
#pragma unroll
    for (int k = 0; k < kSph32NC; ++k) w[k] = 0ull;
#pragma unroll 2
    for (int q = 0; q < mp; ++q) {
      const SphPair32 s = tile[q];
      const u64 d0 = add2(sub2(XH[0], pk2(s.hxy.x, s.hxy.y)), sub2(XL[0], pk2(s.lxy.x, s.lxy.y)));
      const u64 d1 = add2(sub2(XH[1], pk2(s.hxy.z, s.hxy.w)), sub2(XL[1], pk2(s.lxy.z, s.lxy.w)));
      const u64 d2 = add2(sub2(XH[2], pk2(s.hzr.x, s.hzr.y)), sub2(XL[2], pk2(s.lzp.x, s.lzp.y)));
      const u64 dd = fma2(d0, d0, fma2(d1, d1, mul2(d2, d2)));
      float qa, qb;
      upk2(add2(dd, C02), qa, qb);
      float ra = rcp_approx(qa), rb = rcp_approx(qb);
      if (COLL) {
        const int2 sl = tslot[q];
        ra = sl.x == i ? 0.f : ra;
        rb = sl.y == i ? 0.f : rb;
      }
      const u64 r = pk2(ra, rb);
      // sz, ss are twice the pair scalars (the strengths are stored doubled),
      // so R, Q = sz r, ss r; the sums of sz and ss are halved in the epilogue
      const u64 sz = mul2(pk2(s.hzr.z, s.hzr.w), r), ss = mul2(pk2(s.lzp.z, s.lzp.w), r);
      const u64 R = mul2(sz, r), Q = mul2(ss, r);
      w[0] = fma2(sz, d0, w[0]);
      w[1] = fma2(sz, d1, w[1]);
      w[2] = fma2(sz, d2, w[2]);
      w[3] = fma2(ss, d0, w[3]);
      w[4] = fma2(ss, d1, w[4]);
      w[5] = fma2(ss, d2, w[5]);
      const u64 r0 = mul2(R, d0), r1 = mul2(R, d1), r2 = mul2(R, d2);
      const u64 q0 = mul2(Q, d0), q1 = mul2(Q, d1), q2 = mul2(Q, d2);
      w[6] = add2(w[6], r0);
      w[7] = add2(w[7], r1);
      w[8] = add2(w[8], r2);
      w[9] = add2(w[9], q0);
      w[10] = add2(w[10], q1);
      w[11] = add2(w[11], q2);
      w[12] = fma2(r0, d0, w[12]);
      w[13] = fma2(r0, d1, w[13]);
      w[14] = fma2(r0, d2, w[14]);
      w[15] = fma2(r1, d1, w[15]);
      w[16] = fma2(r1, d2, w[16]);
      w[17] = fma2(r2, d2, w[17]);
      w[18] = fma2(q0, d0, w[18]);
      w[19] = fma2(q0, d1, w[19]);
      w[20] = fma2(q0, d2, w[20]);
      w[21] = fma2(q1, d1, w[21]);
      w[22] = fma2(q1, d2, w[22]);
      w[23] = fma2(q2, d2, w[23]);
      w[24] = add2(w[24], sz);
      w[25] = add2(w[25], ss);
      w[26] = fma2(ss, dd, w[26]);
    }
#pragma unroll
    for (int k = 0; k < kSph32NC; ++k) {
      float a, b;
      upk2(w[k], a, b);
      acc[k][tid] += double(a) + double(b);
    }
  }
  if (!valid) return;
#pragma unroll
  for (int k = 0; k < kSph32NC; ++k) part[(c * kSph32NC + k) * tpad + i] = acc[k][tid];
}

__global__ void k_swe_sphere32_out(const double* __restrict__ part, int nchunks, int64_t tpad,
                                   View tx, int64_t nt, double eps2, View u,
                                   double* __restrict__ ddot, double* __restrict__ grad,
                                   int do_velocity) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  double s[kSph32NC];
#pragma unroll
  for (int k = 0; k < kSph32NC; ++k) s[k] = 0.0;
  for (int c = 0; c < nchunks; ++c)
#pragma unroll
    for (int k = 0; k < kSph32NC; ++k) s[k] += part[(int64_t(c) * kSph32NC + k) * tpad + i];
  // the kernel's sz, ss were doubled (strengths stored as rot, pot / pi):
  // halve A, B, Z, G, H (exact)
  for (int k : {0, 1, 2, 3, 4, 5, 24, 25, 26}) s[k] *= 0.5;
  const double x[3] = {tx(i, 0), tx(i, 1), tx(i, 2)};
  const double *A = s, *B = s + 3, *U1 = s + 6, *V1 = s + 9;
  const int sym[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};  // (a, b) -> packed symmetric index
  const double *U2 = s + 12, *V2 = s + 18;
  const double Z = s[24], G = s[25], H = s[26];
  double P[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) P[3 * a + b] = (a == b ? 1.0 : 0.0) - x[a] * x[b];
  auto cross = [](const double* p, const double* q, double* o) {
    o[0] = p[1] * q[2] - p[2] * q[1];
    o[1] = p[2] * q[0] - p[0] * q[2];
    o[2] = p[0] * q[1] - p[1] * q[0];
  };
  if (do_velocity) {
    double ax[3];
    cross(A, x, ax);
#pragma unroll
    for (int a = 0; a < 3; ++a) u(i, a) = ax[a] - (P[3 * a] * B[0] + P[3 * a + 1] * B[1] + P[3 * a + 2] * B[2]);
  }
  double u1x[3], pv1[3], zy[3];
  cross(U1, x, u1x);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    pv1[a] = P[3 * a] * V1[0] + P[3 * a + 1] * V1[1] + P[3 * a + 2] * V1[2];
    zy[a] = Z * x[a] - A[a];
  }
  const double Yx[9] = {0.0, -zy[2], zy[1], zy[2], 0.0, -zy[0], -zy[1], zy[0], 0.0};
  const double g = G - 0.5 * H;
  double M[9];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const double col[3] = {U2[sym[b]], U2[sym[3 + b]], U2[sym[6 + b]]};
    double t1[3];
    cross(col, x, t1);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double v2p = V2[sym[3 * a]] * P[b] + V2[sym[3 * a + 1]] * P[3 + b] + V2[sym[3 * a + 2]] * P[6 + b];
      M[3 * a + b] = eps2 * u1x[a] * x[b] + t1[a] + eps2 * x[a] * pv1[b] + v2p + Yx[3 * a + b] -
                     g * P[3 * a + b];
    }
  }
  double dsum = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) dsum = da(dsum, dm(M[3 * a + b], M[3 * b + a]));
  ddot[i] = dsum;
  if (grad)
#pragma unroll
    for (int k = 0; k < 9; ++k) grad[9 * i + k] = M[k];
}

// Scratch and chunking shared by the four SWE paths: 128 targets per CTA,
// sources compacted (masked slots dropped) and split into chunks of whole
// 256-source tiles, about four waves of CTAs; ncomp FP64 partials per
// (chunk, target), added in fixed order by the epilogue.
struct SwePlan {
  int64_t nb = 0, tpad = 0, ns = 0, chunk_len = 0;
  int nchunks = 1;
  int* src2slot = nullptr;
  void* src = nullptr;     // ns packed source records
  int* slot = nullptr;     // ns slot indices (when asked for)
  double* part = nullptr;  // [chunk][ncomp][tpad]
  dim3 grid() const { return dim3{unsigned(nb), unsigned(nchunks), 1u}; }
};

SwePlan swe_plan(lpm_context& ctx, const uint8_t* mask, int64_t nt, int64_t nf, size_t rec_bytes,
                 int ncomp, bool want_slot) {
  SwePlan p;
  ctx.arena.reset();
  p.nb = (nt + kSweNT - 1) / kSweNT;
  p.tpad = p.nb * kSweNT;
  const int64_t want = std::max<int64_t>(1, (int64_t(ctx.num_sms) * 4 * 8 + p.nb - 1) / p.nb);
  const int64_t nch_max =
      std::max<int64_t>(1, std::min<int64_t>(want, (nf + kSweTile - 1) / kSweTile));
  ctx.arena.reserve(sizeof(int) * (3 * size_t(nf) + 2 * size_t(nf) / 1024 + 8) +
                    rec_bytes * size_t(nf) + sizeof(double) * ncomp * size_t(nch_max) * p.tpad +
                    8 * 4096);
  int* slot2src = static_cast<int*>(ctx.arena.take(sizeof(int) * std::max<int64_t>(nf, 1)));
  p.src2slot = static_cast<int*>(ctx.arena.take(sizeof(int) * std::max<int64_t>(nf, 1)));
  p.ns = compact_sources(ctx, mask, nf, slot2src, p.src2slot);
  // one record more than the sources: the FP32 spherical path packs pairs
  p.src = ctx.arena.take(rec_bytes * size_t(p.ns + 1));
  if (want_slot) p.slot = static_cast<int*>(ctx.arena.take(sizeof(int) * size_t(p.ns + 1)));
  int64_t len = (p.ns + nch_max - 1) / nch_max;
  p.chunk_len = std::max<int64_t>(kSweTile, (len + kSweTile - 1) / kSweTile * kSweTile);
  p.nchunks = int(std::max<int64_t>(1, (p.ns + p.chunk_len - 1) / p.chunk_len));
  p.part = static_cast<double*>(ctx.arena.take(sizeof(double) * ncomp * size_t(p.nchunks) * p.tpad));
  return p;
}

unsigned blocks256(int64_t n) { return unsigned((n + 255) / 256); }

void swe_sphere_sums32(lpm_context& ctx, View tx, int64_t nt, View fx, const double* zeta,
                       const double* sigma, const double* area, const uint8_t* mask, int64_t nf,
                       double eps, bool collocated, View u, double* ddot, double* grad,
                       int do_velocity) {
  // one 64-byte pair record per two sources (32 bytes per source, plus one
  // dummy for an odd count); the pair slots take the plan's slot array
  const SwePlan p = swe_plan(ctx, mask, nt, nf, sizeof(SphPair32) / 2, kSph32NC, true);
  auto* src = static_cast<SphPair32*>(p.src);
  auto* pslot = reinterpret_cast<int2*>(p.slot);
  if (p.ns > 0) {
    k_swe_sphere32_pack<<<blocks256((p.ns + 1) / 2), 256, 0, ctx.stream>>>(
        fx, zeta, sigma, area, p.src2slot, p.ns, src, pslot);
    ctx.launches++;
  }
  const float c0 = float(2 * eps * eps);
  if (collocated)
    k_swe_sphere32<true><<<p.grid(), kSweNT, 0, ctx.stream>>>(tx, nt, src, pslot, p.ns,
                                                              p.chunk_len, c0, p.part, p.tpad);
  else
    k_swe_sphere32<false><<<p.grid(), kSweNT, 0, ctx.stream>>>(tx, nt, src, pslot, p.ns,
                                                               p.chunk_len, c0, p.part, p.tpad);
  k_swe_sphere32_out<<<blocks256(nt), 256, 0, ctx.stream>>>(p.part, p.nchunks, p.tpad, tx, nt,
                                                            eps * eps, u, ddot, grad, do_velocity);
  ctx.launches += 2;
  LPM_CUDA(cudaGetLastError());
}

// Targets tx (nt x 3); sources: face slots fx/zeta/sigma/area/mask (nf);
// collocated: targets are the face slots themselves (i == j skipped).
void swe_sphere_sums(lpm_context& ctx, View tx, int64_t nt, View fx, const double* zeta,
                     const double* sigma, const double* area, const uint8_t* mask, int64_t nf,
                     double eps, bool collocated, View u, double* ddot, double* grad,
                     int do_velocity) {
  if (nt == 0) return;
  if (ctx.precision == LPM_FP32C) {
    swe_sphere_sums32(ctx, tx, nt, fx, zeta, sigma, area, mask, nf, eps, collocated, u, ddot, grad,
                      do_velocity);
    return;
  }
  const SwePlan p = swe_plan(ctx, mask, nt, nf, sizeof(SphSrc), kSphNC, false);
  auto* src = static_cast<SphSrc*>(p.src);
  if (p.ns > 0) {
    k_swe_sphere_pack<<<blocks256(p.ns), 256, 0, ctx.stream>>>(fx, zeta, sigma, area, p.src2slot,
                                                               p.ns, src);
    ctx.launches++;
  }
  k_swe_sphere<<<p.grid(), kSweNT, 0, ctx.stream>>>(tx, nt, src, p.ns, p.chunk_len, eps,
                                                    collocated ? 1 : 0, p.part, p.tpad);
  k_swe_sphere_out<<<blocks256(nt), 256, 0, ctx.stream>>>(p.part, p.nchunks, p.tpad, tx, nt, u,
                                                          ddot, grad, do_velocity);
  ctx.launches += 2;
  LPM_CUDA(cudaGetLastError());
}

bool bad_count(int64_t n) { return n < 0 || n > (int64_t(1) << 31) - 1; }

// FloatingPoint<Real>::zero (src/util/lpm_floating_point.hpp:26-29): |x| < DBL_EPSILON
bool fp_zero(double x) { return std::fabs(x) < 2.220446049250313e-16; }

// Targets tx (nt x 2) with surface ts; sources: face slots fx/zeta/sigma/
// area/mask/sfc (nf); collocated: targets are the face slots themselves.
void swe_plane_sums32(lpm_context& ctx, View tx, const double* ts, int64_t nt, View fx,
                      const double* zeta, const double* sigma, const double* area,
                      const uint8_t* mask, const double* sfc, int64_t nf, double eps,
                      double pse_eps, bool collocated, const SweOut& out) {
  // one 80-byte pair record per two sources (plus one dummy for an odd count)
  const SwePlan p = swe_plan(ctx, mask, nt, nf, sizeof(PlPair32) / 2, kPl32NC, false);
  auto* src = static_cast<PlPair32*>(p.src);
  if (p.ns > 0) {
    k_swe_plane32_pack<<<blocks256((p.ns + 1) / 2), 256, 0, ctx.stream>>>(
        fx, zeta, sigma, area, sfc, p.src2slot, p.ns, src);
    ctx.launches++;
  }
  const float e2 = float(eps * eps), ipse2 = float(1.0 / (pse_eps * pse_eps));
  if (collocated)
    k_swe_plane32<true><<<p.grid(), kSweNT, 0, ctx.stream>>>(tx, ts, nt, src, p.ns, p.chunk_len,
                                                             e2, ipse2, p.part, p.tpad);
  else
    k_swe_plane32<false><<<p.grid(), kSweNT, 0, ctx.stream>>>(tx, ts, nt, src, p.ns, p.chunk_len,
                                                              e2, ipse2, p.part, p.tpad);
  k_swe_plane32_out<<<blocks256(nt), 256, 0, ctx.stream>>>(p.part, p.nchunks, p.tpad, nt, pse_eps,
                                                           out);
  ctx.launches += 2;
  LPM_CUDA(cudaGetLastError());
}

void swe_plane_sums(lpm_context& ctx, View tx, const double* ts, int64_t nt, View fx,
                    const double* zeta, const double* sigma, const double* area,
                    const uint8_t* mask, const double* sfc, int64_t nf, double eps,
                    double pse_eps, bool collocated, const SweOut& out) {
  if (nt == 0) return;
  if (ctx.precision == LPM_FP32C) {
    swe_plane_sums32(ctx, tx, ts, nt, fx, zeta, sigma, area, mask, sfc, nf, eps, pse_eps,
                     collocated, out);
    return;
  }
  const SwePlan p = swe_plan(ctx, mask, nt, nf, sizeof(SweSrc), kSweNC, false);
  auto* src = static_cast<SweSrc*>(p.src);
  if (p.ns > 0) {
    k_swe_pack<<<blocks256(p.ns), 256, 0, ctx.stream>>>(fx, zeta, sigma, area, sfc, p.src2slot,
                                                        p.ns, src);
    ctx.launches++;
  }
  k_swe_plane<<<p.grid(), kSweNT, 0, ctx.stream>>>(tx, ts, nt, src, p.ns, p.chunk_len, eps, pse_eps,
                                                   collocated ? 1 : 0, p.part, p.tpad);
  k_swe_out<<<blocks256(nt), 256, 0, ctx.stream>>>(p.part, p.nchunks, p.tpad, nt, out);
  ctx.launches += 2;
  LPM_CUDA(cudaGetLastError());
}

}  // namespace
}  // namespace lpm

namespace {
int swe_args(lpm_context* ctx, lpm_view u, double* ddot, double* a, double* b, double* c,
             double* d, double* laps, double* psi, double* phi, lpm_view x, const double* s,
             int64_t nt, lpm_view fx, const double* zeta, const double* sigma, const double* area,
             const uint8_t* mask, const double* fs, int64_t nf, double eps, double pse_eps,
             int do_velocity) {
  if (!ctx) return lpm::fail(LPM_ERR_ARG, "null context");
  if (lpm::bad_count(nt) || lpm::bad_count(nf))
    return lpm::fail(LPM_ERR_ARG, "count out of range [0, 2^31-1]");
  if (nt > 0 && (!x.p || !s || !ddot || !a || !b || !c || !d || !laps || !psi || !phi ||
                 (do_velocity && !u.p)))
    return lpm::fail(LPM_ERR_ARG, "null target or output array");
  if (nf > 0 && (!fx.p || !zeta || !sigma || !area || !mask || !fs))
    return lpm::fail(LPM_ERR_ARG, "null source array");
  if (!(eps >= 0) || !std::isfinite(eps) || !(pse_eps > 0) || !std::isfinite(pse_eps))
    return lpm::fail(LPM_ERR_ARG, "eps must be >= 0 and pse_eps > 0, both finite");
  return LPM_OK;
}
}  // namespace

extern "C" {

int lpm_swe_plane_vertex_sums(lpm_context* ctx, lpm_view u, double* ddot, double* du1dx1,
                              double* du1dx2, double* du2dx1, double* du2dx2, double* laps,
                              double* psi, double* phi, lpm_view vx, const double* vs, int64_t nv,
                              lpm_view fx, const double* fzeta, const double* fsigma,
                              const double* farea, const uint8_t* fmask, const double* fs,
                              int64_t nf, double eps, double pse_eps, int do_velocity) {
  if (int r = swe_args(ctx, u, ddot, du1dx1, du1dx2, du2dx1, du2dx2, laps, psi, phi, vx, vs, nv,
                       fx, fzeta, fsigma, farea, fmask, fs, nf, eps, pse_eps, do_velocity))
    return r;
  try {
    lpm::DeviceGuard device_guard(ctx->device);
    lpm::SweOut o{lpm::to_view(u), ddot, du1dx1, du1dx2, du2dx1, du2dx2, laps, psi, phi, do_velocity};
    lpm::swe_plane_sums(*ctx, lpm::to_view(vx), vs, nv, lpm::to_view(fx), fzeta, fsigma, farea,
                        fmask, fs, nf, eps, pse_eps, false, o);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_swe_plane_face_sums(lpm_context* ctx, lpm_view u, double* ddot, double* du1dx1,
                            double* du1dx2, double* du2dx1, double* du2dx2, double* laps,
                            double* psi, double* phi, lpm_view fx, const double* fzeta,
                            const double* fsigma, const double* farea, const uint8_t* fmask,
                            const double* fs, int64_t nf, double eps, double pse_eps,
                            int do_velocity) {
  if (int r = swe_args(ctx, u, ddot, du1dx1, du1dx2, du2dx1, du2dx2, laps, psi, phi, fx, fs, nf,
                       fx, fzeta, fsigma, farea, fmask, fs, nf, eps, pse_eps, do_velocity))
    return r;
  try {
    lpm::DeviceGuard device_guard(ctx->device);
    lpm::SweOut o{lpm::to_view(u), ddot, du1dx1, du1dx2, du2dx1, du2dx2, laps, psi, phi, do_velocity};
    // PlanarSWEFaceSums: collocated = FloatingPoint<Real>::zero(eps)
    lpm::swe_plane_sums(*ctx, lpm::to_view(fx), fs, nf, lpm::to_view(fx), fzeta, fsigma, farea,
                        fmask, fs, nf, eps, pse_eps, lpm::fp_zero(eps), o);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_swe_sphere_vertex_sums(lpm_context* ctx, lpm_view u, double* ddot, double* grad,
                               lpm_view vx, int64_t nv, lpm_view fx, const double* fzeta,
                               const double* fsigma, const double* farea, const uint8_t* fmask,
                               int64_t nf, double eps, int do_velocity) {
  if (!ctx) return lpm::fail(LPM_ERR_ARG, "null context");
  if (lpm::bad_count(nv) || lpm::bad_count(nf))
    return lpm::fail(LPM_ERR_ARG, "count out of range [0, 2^31-1]");
  if (nv > 0 && (!vx.p || !ddot || (do_velocity && !u.p)))
    return lpm::fail(LPM_ERR_ARG, "null target or output array");
  if (nf > 0 && (!fx.p || !fzeta || !fsigma || !farea || !fmask))
    return lpm::fail(LPM_ERR_ARG, "null source array");
  if (!(eps >= 0) || !std::isfinite(eps)) return lpm::fail(LPM_ERR_ARG, "eps must be finite and >= 0");
  try {
    lpm::DeviceGuard device_guard(ctx->device);
    lpm::swe_sphere_sums(*ctx, lpm::to_view(vx), nv, lpm::to_view(fx), fzeta, fsigma, farea, fmask,
                         nf, eps, false, lpm::to_view(u), ddot, grad, do_velocity);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_swe_sphere_face_sums(lpm_context* ctx, lpm_view u, double* ddot, double* grad,
                             lpm_view fx, const double* fzeta, const double* fsigma,
                             const double* farea, const uint8_t* fmask, int64_t nf, double eps,
                             int do_velocity) {
  if (!ctx) return lpm::fail(LPM_ERR_ARG, "null context");
  if (lpm::bad_count(nf)) return lpm::fail(LPM_ERR_ARG, "count out of range [0, 2^31-1]");
  if (nf > 0 && (!fx.p || !fzeta || !fsigma || !farea || !fmask || !ddot || (do_velocity && !u.p)))
    return lpm::fail(LPM_ERR_ARG, "null input or output array");
  if (!(eps >= 0) || !std::isfinite(eps)) return lpm::fail(LPM_ERR_ARG, "eps must be finite and >= 0");
  try {
    lpm::DeviceGuard device_guard(ctx->device);
    // SphereFaceSums: collocated = FloatingPoint<Real>::zero(eps)
    lpm::swe_sphere_sums(*ctx, lpm::to_view(fx), nf, lpm::to_view(fx), fzeta, fsigma, farea, fmask,
                         nf, eps, lpm::fp_zero(eps), lpm::to_view(u), ddot, grad, do_velocity);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

}  // extern "C"

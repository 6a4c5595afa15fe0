// nbody.cuh -- tiled direct-summation kernels for sm_103a.
//
// One CTA owns NT*R targets (R per thread, held in registers) and one chunk
// of the packed source array.  The chunk streams through shared memory in
// tiles of TILE sources, double-buffered: one elected thread issues a bulk
// asynchronous copy (cp.async.bulk, the TMA engine) per tile and the CTA waits
// on an mbarrier with a bounded spin.  Every thread reads each source record
// as a shared-memory broadcast and applies it to its R targets.  Each CTA
// writes one FP64 partial per (chunk, component, target); a combine kernel
// adds the chunks in fixed order, so results are deterministic.
//
// FP32 path (the fast form).  With d = x - y and q = |d|^2 + c0:
//   sphere: 1 - x.y + eps^2 = q/2 for unit vectors, c0 = 2 eps^2;
//           x cross y = d cross x, so
//           u_i = -(1/2pi) (sum_j (g_j/q_j) d_j) cross x_i,
//           psi_i = -(ln2/4pi) (sum_j g_j lg2 q_j - sum_j g_j)
//   plane:  c0 = eps^2, u = (-w_1, w_0)/(2pi), psi = -(ln2/4pi) sum g lg2 q
// with g = zeta*area and w = sum (g/q) d.  Hoisting the cross product out of
// the sum leaves 10 FP32 operations and one MUFU reciprocal per pair.  c0
// also carries a 1e-30 floor so a coincident pair (d = 0, the skipped i == j
// term) contributes exactly 0 to w.  Sums are kept as (S, C) pairs: each
// tile's plain FP32 partial is merged with an error-free TwoSum, so the
// compensation costs O(1/TILE) per pair.
//
// FP64 path (LPM_FP64, parity form within 1e-12).  The reference's kernels
// (1 - x.y [+ eps^2] on the sphere, |x - y|^2 + eps^2 on the plane) with the
// cross product hoisted out of the sum: per target B = sum_j (g_j / arg_j) y_j
// and u = s (x cross B) in the epilogue; one quotient per pair by Newton's
// method from the hardware's approximate reciprocal.  11 FP64 operations per
// sphere pair (eps form), against ~32 with three correctly rounded divisions.
//
// FP64 exact path (LPM_FP64_EXACT).  Every pair term is computed with the
// reference's formula and operation order using non-contracting intrinsics
// (__dmul_rn/__dadd_rn/__ddiv_rn), so each term equals the reference's term
// bit for bit; only the grouping of the sum differs.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

#include <cuda_runtime.h>

#include "f32x2.cuh"
#include "lpm_gb300.h"

namespace lpm {

constexpr double kPI = 3.1415926535897932384626433832795;
constexpr double kFOURPI = 4 * kPI;     // 4 * constants::PI
constexpr double kNEGFOURPI = -4 * kPI;  // -4 * constants::PI
constexpr double kTWOPI = 2 * kPI;       // 2 * constants::PI
constexpr float kQFLOOR = 1e-30f;

// Bounded spin limit for mbarrier waits (each try_wait may also suspend in
// hardware), roughly a second at worst before giving up.
constexpr unsigned kSpinLimit = 1u << 24;

// ---------------------------------------------------------------------------
// PTX helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
// Bulk (non-tensor) TMA copy global -> shared, completion on an mbarrier.
// dst/src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src,
                                            unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Returns false if the phase did not complete within `limit` tries.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity,
                                                  unsigned limit = kSpinLimit) {
  for (unsigned it = 0; it < limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}

// Error-free transformation a + b = s + e (Knuth TwoSum), accumulated into
// the compensation term.
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float p) {
  const float t = s + p;
  const float bp = t - s;
  const float e = (s - (t - bp)) + (p - bp);
  s = t;
  c += e;
}

// ---------------------------------------------------------------------------
// Tile pipeline shared by both precisions.
// ---------------------------------------------------------------------------
template <typename Rec, int TILE>
struct TilePipe {
  Rec* buf;        // [2][TILE] in shared memory
  uint64_t* bar;   // [2]
  const Rec* src;  // chunk start in global memory
  int ntiles;
  unsigned g0 = 0;  // tiles this CTA consumed before the chunk (a persistent
                    // CTA keeps the barriers' phases running across chunks)
  unsigned spin = kSpinLimit;  // polls per wait before giving up

  __device__ void init() {
    if (threadIdx.x == 0) {
      mbar_init(&bar[0], 1);
      mbar_init(&bar[1], 1);
      mbar_fence_init();
    }
    __syncthreads();
  }
  __device__ void prefetch() {
    if (threadIdx.x == 0) {
      for (int t = 0; t < 2 && t < ntiles; ++t) issue(t);
    }
  }
  __device__ void start() {
    init();
    prefetch();
  }
  __device__ void issue(int t) {
    const unsigned b = (g0 + t) & 1;
    const unsigned bytes = TILE * sizeof(Rec);
    mbar_expect_tx(&bar[b], bytes);
    tma_load_1d(buf + b * TILE, src + (int64_t)t * TILE, bytes, &bar[b]);
  }
  // Waits for tile t; returns false (CTA-uniform) if the wait gave up.
  __device__ bool acquire(int t) {
    const unsigned g = g0 + t;
    const bool ok = mbar_wait_bounded(&bar[g & 1], (g >> 1) & 1, spin);
    return !__syncthreads_or(!ok);
  }
  // All threads are done with tile t: refill its buffer with tile t + 2.
  __device__ void release(int t) {
    __syncthreads();
    if (threadIdx.x == 0 && t + 2 < ntiles) issue(t + 2);
  }
  // After a timeout: wait (bounded) for copies still in flight, then return.
  __device__ void drain(int t, int* err) {
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      for (int k = t; k < t + 2 && k < ntiles; ++k) {
        const unsigned g = g0 + k;
        (void)mbar_wait_bounded(&bar[g & 1], (g >> 1) & 1, spin);
      }
    }
  }
  __device__ const Rec* tile(int t) const { return buf + ((g0 + t) & 1) * TILE; }
};

// ---------------------------------------------------------------------------
// Chord-form kernel, FP32 (LPM_FP32C) or FP64 (LPM_FP64_CHORD).
//   tgt: vec4 (x, y, z, g_self) per target, ntgt_pad entries
//   src: vec4 (x, y, z, g) per source (plane: z = 0), nsrc_pad entries
//   part: [chunk][comp][ntgt_pad] doubles; comps = (WU ? NDIM : 0) +
//         (WP ? 1 : 0): (w0 w1 [w2] [L]) with L = sum g lg2 q
// FP32 uses the MUFU reciprocal and log2; FP64 divides and calls log2.
// ---------------------------------------------------------------------------
template <typename T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4_16a; };

// FP32 source record with every value duplicated, (x, x, y, y) (z, z, g, g),
// so that the packed f32x2 instructions apply one source to two targets
// without re-packing it per pair.
struct __align__(16) SrcF32 {
  float4 a, b;
};
__host__ __device__ inline SrcF32 make_src_f32(float x, float y, float z, float g) {
  return SrcF32{make_float4(x, x, y, y), make_float4(z, z, g, g)};
}
template <typename T> struct SrcRec;
template <> struct SrcRec<float> { using type = SrcF32; };
template <> struct SrcRec<double> { using type = double4_16a; };

__device__ __forceinline__ float chord_rcp(float q) { return rcp_approx(q); }
__device__ __forceinline__ double chord_rcp(double q) { return 1.0 / q; }
__device__ __forceinline__ float chord_lg2(float q) { return lg2_approx(q); }
__device__ __forceinline__ double chord_lg2(double q) { return log2(q); }
__device__ __forceinline__ float chord_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double chord_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ void two_sum_acc(double& s, double& c, double p) {
  const double t = s + p;
  const double bp = t - s;
  const double e = (s - (t - bp)) + (p - bp);
  s = t;
  c += e;
}

// Which sources (bit k: source index = k mod 8) take their reciprocal from
// Newton's method on the FMA pipe instead of the MUFU: the planar kernel with
// velocity and stream function needs two MUFU results per pair (reciprocal,
// log2), and a MUFU result holds the XU pipe two cycles (16 per clock per SM),
// while the pair's 8 FP32 lane operations leave half of the FP32 pipe (128
// lanes per clock per SM) idle.  The Newton reciprocal costs 6 FP32 lane
// operations (3 packed FMAs) and one integer operation.  Measured on the
// planar RK2 step (quad level 9), against the MUFU for every source: 1
// source in 8 +4.3 %, 2 in 8 +8 %, 3 in 8 +9.4 %, 4 in 8 +4.8 %, 6 in 8 -2 %
// (the issue slots the Newton steps take count as well).
// The choice depends on the source's index alone (tiles and chunks start at
// multiples of 8), so a target's sums do not depend on the kernel shape or the
// chunking.  The velocity-only kernels keep the MUFU for every source.
__host__ __device__ constexpr unsigned soft_rcp_sources(int ndim, bool wu, bool wp) {
  return (ndim == 2 && wu && wp) ? 0x25u : 0u;
}

// -1/q for a packed pair of positive normal floats, by Newton's method on the
// negated reciprocal y (y <- y + y (1 + q y), two FMAs, no negation) from the
// bit-level initial approximation -1/q ~ bits(0xFEF311C3 - bits(q)) (the
// classic integer reciprocal seed, relative error <= 5.1 %): three steps take
// it to <= 0.5 ulp (6e-8 relative), tested against FP64 1/q.
__device__ __forceinline__ u64 neg_rcp2(u64 q, float qa, float qb, u64 one2) {
  u64 y = pk2(__uint_as_float(0xFEF311C3u - __float_as_uint(qa)),
              __uint_as_float(0xFEF311C3u - __float_as_uint(qb)));
#pragma unroll
  for (int it = 0; it < 3; ++it) y = fma2(y, fma2(q, y, one2), y);
  return y;
}

// One source record against the thread's H packed target pairs (FP32 chord
// form, velocity and stream function); SOFT: the reciprocal by neg_rcp2.
template <bool SOFT, int NDIM, bool SKIPC, int H, int NC, typename Rec>
__device__ __forceinline__ void chord_pair_up(const Rec& s, const u64 (&TX)[H], const u64 (&TY)[H],
                                              const u64 (&TZ)[H], u64 C02, float c0, u64 one2,
                                              u64 (&P)[NC][H]) {
  const u64 sx = pk2(s.a.x, s.a.y), sy = pk2(s.a.z, s.a.w);
  const u64 sz = pk2(s.b.x, s.b.y), sw = pk2(s.b.z, s.b.w);
  u64 nsw = 0ull;
  if constexpr (SOFT) nsw = fma2(sw, pk2(-1.f, -1.f), 0ull);  // -g, exact
#pragma unroll
  for (int h = 0; h < H; ++h) {
    const u64 dx = sub2(TX[h], sx);
    const u64 dy = sub2(TY[h], sy);
    u64 dz = 0ull;
    u64 q;
    if (NDIM == 3) {
      dz = sub2(TZ[h], sz);
      q = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, C02)));
    } else {
      q = fma2(dx, dx, fma2(dy, dy, C02));
    }
    float qa, qb;
    upk2(q, qa, qb);
    u64 w;
    if constexpr (SOFT)
      w = mul2(nsw, neg_rcp2(q, qa, qb, one2));
    else
      w = mul2(sw, pk2(rcp_approx(qa), rcp_approx(qb)));
    P[0][h] = fma2(w, dx, P[0][h]);
    P[1][h] = fma2(w, dy, P[1][h]);
    if (NDIM == 3) P[2][h] = fma2(w, dz, P[2][h]);
    float la = lg2_approx(qa), lb = lg2_approx(qb);
    if (SKIPC) {
      la = (qa == c0) ? 0.f : la;
      lb = (qb == c0) ? 0.f : lb;
    }
    P[NC - 1][h] = fma2(sw, pk2(la, lb), P[NC - 1][h]);
  }
}

// Eight consecutive sources, each with its compile-time reciprocal choice.
template <unsigned PAT, int NDIM, bool SKIPC, int H, int NC, typename Rec, size_t... J>
__device__ __forceinline__ void chord_group8_up(const Rec* sm, const u64 (&TX)[H],
                                                const u64 (&TY)[H], const u64 (&TZ)[H], u64 C02,
                                                float c0, u64 one2, u64 (&P)[NC][H],
                                                std::index_sequence<J...>) {
  (chord_pair_up<((PAT >> J) & 1u) != 0, NDIM, SKIPC, H, NC>(sm[J], TX, TY, TZ, C02, c0, one2,
                                                             P),
   ...);
}

// SKIPC: in the stream-function sum, drop coincident pairs (q == c0, i.e.
// d == 0: the skipped i == j term).  The velocity term of such a pair is 0.
template <typename T, int NDIM, bool WU, bool WP>
struct ChordAcc {
  static constexpr int NC = (WU ? NDIM : 0) + (WP ? 1 : 0);
};

// Runs one chunk (pipe.ntiles tiles already prefetched) for R targets per
// thread, accumulating into the compensated sums (S, C).  Returns false if a
// tile wait gave up (the pipe has been drained and err set).
//
// FP32: targets are processed in pairs (2h, 2h+1) with f32x2 instructions
// against the duplicated source record: 5 packed FP32 instructions and one
// MUFU reciprocal per pair instead of 10 scalar ones.  Each packed operation
// is the two scalar operations, so the results are those of the scalar form.
template <typename T, int NDIM, bool WU, bool WP, bool SKIPC, int R, int TILE>
__device__ __forceinline__ bool chord_chunk(
    TilePipe<typename SrcRec<T>::type, TILE>& pipe, const T (&tx)[R], const T (&ty)[R],
    const T (&tz)[R], T (&S)[ChordAcc<T, NDIM, WU, WP>::NC][R],
    T (&C)[ChordAcc<T, NDIM, WU, WP>::NC][R], T c0, int* err) {
  using Rec = typename SrcRec<T>::type;
  constexpr int NC = ChordAcc<T, NDIM, WU, WP>::NC;
  if constexpr (std::is_same<T, float>::value) {
    static_assert(R % 2 == 0, "packed FP32 needs an even number of targets per thread");
    constexpr int H = R / 2;
    u64 TX[H], TY[H], TZ[H];
#pragma unroll
    for (int h = 0; h < H; ++h) {
      TX[h] = pk2(tx[2 * h], tx[2 * h + 1]);
      TY[h] = pk2(ty[2 * h], ty[2 * h + 1]);
      TZ[h] = pk2(tz[2 * h], tz[2 * h + 1]);
    }
    const u64 C02 = pk2(c0, c0);
    for (int t = 0; t < pipe.ntiles; ++t) {
      if (!pipe.acquire(t)) {
        pipe.drain(t, err);
        return false;
      }
      const Rec* sm = pipe.tile(t);
      u64 P[NC][H];
#pragma unroll
      for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int h = 0; h < H; ++h) P[k][h] = 0ull;

      constexpr unsigned kSoft = soft_rcp_sources(NDIM, WU, WP);
      if constexpr (kSoft != 0) {
        static_assert(TILE % 8 == 0, "the soft-reciprocal pattern repeats every 8 sources");
        const u64 one2 = pk2(1.f, 1.f);
#pragma unroll 1
        for (int j0 = 0; j0 < TILE; j0 += 8)
          chord_group8_up<kSoft, NDIM, SKIPC, H, NC>(sm + j0, TX, TY, TZ, C02, c0, one2, P,
                                                     std::make_index_sequence<8>{});
      } else {
#pragma unroll 4
      for (int j = 0; j < TILE; ++j) {
        const Rec s = sm[j];
        const u64 sx = pk2(s.a.x, s.a.y), sy = pk2(s.a.z, s.a.w);
        const u64 sz = pk2(s.b.x, s.b.y), sw = pk2(s.b.z, s.b.w);
#pragma unroll
        for (int h = 0; h < H; ++h) {
          const u64 dx = sub2(TX[h], sx);
          const u64 dy = sub2(TY[h], sy);
          u64 dz = 0ull;
          u64 q;
          if (NDIM == 3) {
            dz = sub2(TZ[h], sz);
            q = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, C02)));
          } else {
            q = fma2(dx, dx, fma2(dy, dy, C02));
          }
          float qa, qb;
          upk2(q, qa, qb);
          if (WU) {
            const u64 w = mul2(sw, pk2(rcp_approx(qa), rcp_approx(qb)));
            P[0][h] = fma2(w, dx, P[0][h]);
            P[1][h] = fma2(w, dy, P[1][h]);
            if (NDIM == 3) P[2][h] = fma2(w, dz, P[2][h]);
          }
          if (WP) {
            float la = lg2_approx(qa), lb = lg2_approx(qb);
            if (SKIPC) {
              la = (qa == c0) ? 0.f : la;
              lb = (qb == c0) ? 0.f : lb;
            }
            P[NC - 1][h] = fma2(sw, pk2(la, lb), P[NC - 1][h]);
          }
        }
      }
      }
#pragma unroll
      for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int h = 0; h < H; ++h) {
          float pa, pb;
          upk2(P[k][h], pa, pb);
          two_sum_acc(S[k][2 * h], C[k][2 * h], pa);
          two_sum_acc(S[k][2 * h + 1], C[k][2 * h + 1], pb);
        }
      pipe.release(t);
    }
    return true;
  } else {
    for (int t = 0; t < pipe.ntiles; ++t) {
      if (!pipe.acquire(t)) {
        pipe.drain(t, err);
        return false;
      }
      const Rec* sm = pipe.tile(t);
      T P[NC][R];
#pragma unroll
      for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int r = 0; r < R; ++r) P[k][r] = T(0);

#pragma unroll 4
      for (int j = 0; j < TILE; ++j) {
        const Rec s = sm[j];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const T dx = tx[r] - s.x;
          const T dy = ty[r] - s.y;
          T q;
          T dz = T(0);
          if (NDIM == 3) {
            dz = tz[r] - s.z;
            q = chord_fma(dx, dx, chord_fma(dy, dy, chord_fma(dz, dz, c0)));
          } else {
            q = chord_fma(dx, dx, chord_fma(dy, dy, c0));
          }
          if (WU) {
            const T w = s.w * chord_rcp(q);
            P[0][r] = chord_fma(w, dx, P[0][r]);
            P[1][r] = chord_fma(w, dy, P[1][r]);
            if (NDIM == 3) P[2][r] = chord_fma(w, dz, P[2][r]);
          }
          if (WP) {
            T lg = chord_lg2(q);
            if (SKIPC) lg = (q == c0) ? T(0) : lg;
            P[NC - 1][r] = chord_fma(s.w, lg, P[NC - 1][r]);
          }
        }
      }
#pragma unroll
      for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int r = 0; r < R; ++r) two_sum_acc(S[k][r], C[k][r], P[k][r]);
      pipe.release(t);
    }
    return true;
  }
}

template <typename T, int NDIM, bool WU, bool WP, bool SKIPC, int R, int NT, int TILE,
          int MINB>
__global__ void __launch_bounds__(NT, MINB)
    nbody_chord(const typename Vec4<T>::type* __restrict__ tgt,
                const typename SrcRec<T>::type* __restrict__ src, int64_t ntgt_pad,
                int64_t nsrc_pad, int chunk_len, T c0, double* __restrict__ part,
                int* err) {
  using V4 = typename Vec4<T>::type;
  using Rec = typename SrcRec<T>::type;
  constexpr int NC = ChordAcc<T, NDIM, WU, WP>::NC;
  __shared__ __align__(128) Rec sbuf[2 * TILE];
  __shared__ __align__(8) uint64_t sbar[2];

  const int tid = threadIdx.x;
  const int64_t tbase = (int64_t)blockIdx.x * (NT * R);
  const int64_t s0 = (int64_t)blockIdx.y * chunk_len;
  int64_t slen = nsrc_pad - s0;
  if (slen > chunk_len) slen = chunk_len;

  T tx[R], ty[R], tz[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const V4 t = tgt[tbase + r * NT + tid];
    tx[r] = t.x;
    ty[r] = t.y;
    tz[r] = t.z;
  }
  T S[NC][R], C[NC][R];
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      S[k][r] = T(0);
      C[k][r] = T(0);
    }

  TilePipe<Rec, TILE> pipe{sbuf, sbar, src + s0, int(slen / TILE)};
  pipe.start();
  if (!chord_chunk<T, NDIM, WU, WP, SKIPC, R, TILE>(pipe, tx, ty, tz, S, C, c0, err)) return;

  double* out = part + (int64_t)blockIdx.y * NC * ntgt_pad;
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r)
      out[k * ntgt_pad + tbase + r * NT + tid] =
          (double)S[k][r] + (double)C[k][r];
}

// ---------------------------------------------------------------------------
// FP64 parity kernel.
//   tgt:  double4_16a (x, y, z, unused) per target
//   tself: per-target source index to skip (-1 = none)
//   src:  double4_16a (x, y, z, g): g = (-zeta)*area for FORM_BVE (the reference's
//         circ), zeta*area otherwise
//   part: [chunk][comp][ntgt_pad]; comps = (WU ? NDIM : 0) + (WP ? 1 : 0)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dmul(double a, double b) {
  return __dmul_rn(a, b);
}
__device__ __forceinline__ double dadd(double a, double b) {
  return __dadd_rn(a, b);
}
__device__ __forceinline__ double dsub(double a, double b) {
  return __dsub_rn(a, b);
}
__device__ __forceinline__ double ddiv(double a, double b) {
  return __ddiv_rn(a, b);
}

template <int FORM, bool WU, bool WP, int R, int NT, int TILE>
__global__ void __launch_bounds__(NT)
    nbody_f64(const double4_16a* __restrict__ tgt, const int* __restrict__ tself,
              const double4_16a* __restrict__ src, int64_t ntgt_pad,
              int64_t nsrc_pad, int chunk_len, double eps2,
              double* __restrict__ part, int* err) {
  constexpr int ND = (FORM == 2) ? 2 : 3;
  constexpr int NC = (WU ? ND : 0) + (WP ? 1 : 0);
  __shared__ __align__(128) double4_16a sbuf[2 * TILE];
  __shared__ __align__(8) uint64_t sbar[2];

  const int tid = threadIdx.x;
  const int64_t tbase = (int64_t)blockIdx.x * (NT * R);
  const int64_t s0 = (int64_t)blockIdx.y * chunk_len;
  int64_t slen = nsrc_pad - s0;
  if (slen > chunk_len) slen = chunk_len;

  double x0[R], x1[R], x2[R];
  int self[R];
  double A[NC][R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int64_t ti = tbase + r * NT + tid;
    const double4_16a t = tgt[ti];
    x0[r] = t.x;
    x1[r] = t.y;
    x2[r] = t.z;
    self[r] = tself[ti];
#pragma unroll
    for (int k = 0; k < NC; ++k) A[k][r] = 0.0;
  }

  TilePipe<double4_16a, TILE> pipe{sbuf, sbar, src + s0, int(slen / TILE)};
  pipe.start();
  for (int t = 0; t < pipe.ntiles; ++t) {
    if (!pipe.acquire(t)) {
      pipe.drain(t, err);
      return;
    }
    const double4_16a* sm = pipe.tile(t);
    const int jbase = int(s0 + (int64_t)t * TILE);
#pragma unroll 1
    for (int j = 0; j < TILE; ++j) {
      const double4_16a s = sm[j];
      const int jg = jbase + j;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const bool skip = (jg == self[r]);
        if (FORM == 0) {
          // biot_savart / greens_fn (src/lpm_sphere_functions.hpp:21-57)
          const double dt =
              dadd(dadd(dmul(x0[r], s.x), dmul(x1[r], s.y)), dmul(x2[r], s.z));
          const double omd = dsub(1.0, dt);
          if (WU) {
            const double c0 = dsub(dmul(x1[r], s.z), dmul(x2[r], s.y));
            const double c1 = dsub(dmul(x2[r], s.x), dmul(x0[r], s.z));
            const double c2 = dsub(dmul(x0[r], s.y), dmul(x1[r], s.x));
            const double st = ddiv(s.w, dmul(kFOURPI, omd));
            A[0][r] = dadd(A[0][r], skip ? 0.0 : dmul(c0, st));
            A[1][r] = dadd(A[1][r], skip ? 0.0 : dmul(c1, st));
            A[2][r] = dadd(A[2][r], skip ? 0.0 : dmul(c2, st));
          }
          if (WP) {
            const double p = ddiv(dmul(log(omd), s.w), kFOURPI);
            A[NC - 1][r] = dadd(A[NC - 1][r], skip ? 0.0 : p);
          }
        } else if (FORM == 1) {
          // Incompressible2DKernels<SphereGeometry>::kernel_vals
          // (src/lpm_incompressible2d_kernels.hpp:35-47)
          const double dt =
              dadd(dadd(dmul(x0[r], s.x), dmul(x1[r], s.y)), dmul(x2[r], s.z));
          const double arg = dadd(dsub(1.0, dt), eps2);
          if (WU) {
            const double den = dmul(kNEGFOURPI, arg);
            const double c0 = dsub(dmul(x1[r], s.z), dmul(x2[r], s.y));
            const double c1 = dsub(dmul(x2[r], s.x), dmul(x0[r], s.z));
            const double c2 = dsub(dmul(x0[r], s.y), dmul(x1[r], s.x));
            A[0][r] = dadd(A[0][r], skip ? 0.0 : dmul(ddiv(c0, den), s.w));
            A[1][r] = dadd(A[1][r], skip ? 0.0 : dmul(ddiv(c1, den), s.w));
            A[2][r] = dadd(A[2][r], skip ? 0.0 : dmul(ddiv(c2, den), s.w));
          }
          if (WP) {
            const double p = dmul(ddiv(-log(arg), kFOURPI), s.w);
            A[NC - 1][r] = dadd(A[NC - 1][r], skip ? 0.0 : p);
          }
        } else {
          // Incompressible2DKernels<PlaneGeometry>::kernel_vals (:72-84)
          const double m0 = dsub(x0[r], s.x);
          const double m1 = dsub(x1[r], s.y);
          const double arg = dadd(dadd(dmul(m0, m0), dmul(m1, m1)), eps2);
          if (WU) {
            const double den = dmul(kTWOPI, arg);
            A[0][r] = dadd(A[0][r], skip ? 0.0 : dmul(ddiv(-m1, den), s.w));
            A[1][r] = dadd(A[1][r], skip ? 0.0 : dmul(ddiv(m0, den), s.w));
          }
          if (WP) {
            const double p = dmul(ddiv(-log(arg), kFOURPI), s.w);
            A[NC - 1][r] = dadd(A[NC - 1][r], skip ? 0.0 : p);
          }
        }
      }
    }
    pipe.release(t);
  }

  double* out = part + (int64_t)blockIdx.y * NC * ntgt_pad;
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r) out[k * ntgt_pad + tbase + r * NT + tid] = A[k][r];
}

// ---------------------------------------------------------------------------
// FP64 kernel, cross product hoisted (LPM_FP64).
//   tgt, tself, src: as nbody_f64.
//   sphere forms (FORM 0 = BVE, g = (-zeta) A, eps = 0; FORM 1 = eps kernel,
//   g = zeta A): arg_j = (1 - x.y_j) + eps^2,
//     partials  B = sum_j (g_j / arg_j) y_j   [WU, 3 components]
//               L = sum_j g_j log(arg_j)      [WP]
//   and ref64_epilogue forms u = s (x cross B), psi = s L with s = 1/(4 pi)
//   (BVE: biot_savart, greens_fn) or -1/(4 pi) (kernel_vals).
//   plane (FORM 2): m = x - y_j, arg_j = (m.m) + eps^2,
//     A = sum_j (g_j / arg_j) (-m_1, m_0),  L = sum_j g_j log(arg_j),
//   u = A / (2 pi), psi = -L / (4 pi).
// The skipped pair (i == j) is selected out, so a non-finite quotient of a
// coincident pair never enters the sum.
// ---------------------------------------------------------------------------

// n / d from the PTX approximate FP64 reciprocal r (relative error e0 of
// about 2^-20 or less): with e = 1 - d r (exact to rounding, one fused
// multiply-add), n / d = n r / (1 - e) = n r (1 + e + e^2) + O(e0^3), so
// q = q0 + q0 (e + e^2), q0 = n r -- the second-order Newton-Raphson
// (Halley-type) correction of the quotient, four FP64 operations.  Within
// about one ulp of n / d for the finite, normal d that occur here; d = 0
// gives NaN.
__device__ __forceinline__ double div_nr(double n, double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  const double q0 = n * r;
  const double e = fma(-d, r, 1.0);
  return fma(q0, fma(e, e, e), q0);
}

template <int FORM, bool WU, bool WP, int R, int NT, int TILE>
__global__ void __launch_bounds__(NT)
    nbody_f64h(const double4_16a* __restrict__ tgt, const int* __restrict__ tself,
               const double4_16a* __restrict__ src, int64_t ntgt_pad,
               int64_t nsrc_pad, int chunk_len, double eps2,
               double* __restrict__ part, int* err) {
  constexpr int ND = (FORM == 2) ? 2 : 3;
  constexpr int NC = (WU ? ND : 0) + (WP ? 1 : 0);
  __shared__ __align__(128) double4_16a sbuf[2 * TILE];
  __shared__ __align__(8) uint64_t sbar[2];

  const int tid = threadIdx.x;
  const int64_t tbase = (int64_t)blockIdx.x * (NT * R);
  const int64_t s0 = (int64_t)blockIdx.y * chunk_len;
  int64_t slen = nsrc_pad - s0;
  if (slen > chunk_len) slen = chunk_len;

  double x0[R], x1[R], x2[R];
  int self[R];
  double A[NC][R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int64_t ti = tbase + r * NT + tid;
    const double4_16a t = tgt[ti];
    x0[r] = t.x;
    x1[r] = t.y;
    x2[r] = t.z;
    self[r] = tself[ti];
#pragma unroll
    for (int k = 0; k < NC; ++k) A[k][r] = 0.0;
  }

  TilePipe<double4_16a, TILE> pipe{sbuf, sbar, src + s0, int(slen / TILE)};
  pipe.start();
  for (int t = 0; t < pipe.ntiles; ++t) {
    if (!pipe.acquire(t)) {
      pipe.drain(t, err);
      return;
    }
    const double4_16a* sm = pipe.tile(t);
    const int jbase = int(s0 + (int64_t)t * TILE);
#pragma unroll 2
    for (int j = 0; j < TILE; ++j) {
      const double4_16a s = sm[j];
      const int jg = jbase + j;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const bool skip = (jg == self[r]);
        double arg;
        double m0 = 0.0, m1 = 0.0;
        if (FORM == 2) {
          m0 = x0[r] - s.x;
          m1 = x1[r] - s.y;
          arg = fma(m0, m0, fma(m1, m1, eps2));
        } else {
          // x.y - 1 accumulated from the -1 on, so 1 - x.y [+ eps^2] costs
          // no separate subtraction
          const double dm1 = fma(x2[r], s.z, fma(x1[r], s.y, fma(x0[r], s.x, -1.0)));
          arg = (FORM == 1) ? eps2 - dm1 : -dm1;
        }
        if (WU) {
          const double q = div_nr(s.w, arg);
          const double g = skip ? 0.0 : q;
          if (FORM == 2) {
            A[0][r] = fma(-m1, g, A[0][r]);
            A[1][r] = fma(m0, g, A[1][r]);
          } else {
            A[0][r] = fma(g, s.x, A[0][r]);
            A[1][r] = fma(g, s.y, A[1][r]);
            A[2][r] = fma(g, s.z, A[2][r]);
          }
        }
        if (WP) {
          const double l = fma(log(arg), s.w, A[NC - 1][r]);
          A[NC - 1][r] = skip ? A[NC - 1][r] : l;
        }
      }
    }
    pipe.release(t);
  }

  double* out = part + (int64_t)blockIdx.y * NC * ntgt_pad;
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r) out[k * ntgt_pad + tbase + r * NT + tid] = A[k][r];
}

// Epilogue of the hoisted FP64 kernel for one target: a = summed partials,
// p = the FP64 position the target was evaluated at, form = FORM_*.
template <int NDIM, bool WU, bool WP>
__device__ __forceinline__ void ref64_epilogue(const double* a, const double* p, int form,
                                               double* u, double* psi) {
  constexpr int NC = (WU ? NDIM : 0) + (WP ? 1 : 0);
  constexpr double INV4PI = 1.0 / (4.0 * kPI);
  constexpr double INV2PI = 1.0 / (2.0 * kPI);
  if (NDIM == 3) {
    const double s = form == 0 ? INV4PI : -INV4PI;
    if (WU) {
      u[0] = s * (p[1] * a[2] - p[2] * a[1]);
      u[1] = s * (p[2] * a[0] - p[0] * a[2]);
      u[2] = s * (p[0] * a[1] - p[1] * a[0]);
    }
    if (WP) *psi = s * a[NC - 1];
  } else {
    if (WU) {
      u[0] = INV2PI * a[0];
      u[1] = INV2PI * a[1];
    }
    if (WP) *psi = -INV4PI * a[NC - 1];
  }
}

// Arithmetic modes of the pair sum.
enum Mode : int {
  M_REF64 = 0,  // LPM_FP64 / LPM_FP64_EXACT: the reference's formulas, FP64
  M_C32 = 1,    // LPM_FP32C: chord form, FP32 pairs, compensated sums
  M_C64 = 2     // LPM_FP64_CHORD: chord form, FP64
};
__host__ __device__ inline int mode_of(int precision) {
  return precision == LPM_FP32C ? M_C32 : (precision == LPM_FP64_CHORD ? M_C64 : M_REF64);
}
// LPM_FP64 runs the hoisted kernel; LPM_FP64_EXACT the term-by-term kernel.
__host__ __device__ inline bool ref64_exact(int precision) {
  return precision == LPM_FP64_EXACT;
}

// Chord-form epilogue of one target: a = summed partials (w [, L]), p = the
// FP64 position the target was evaluated at, gs = strength of its skipped
// self source (0 if none), sg = sum of all source strengths (sphere psi).
// c0 is unused (kept for the signature of both modes).
template <int MODE, int NDIM, bool WU, bool WP>
__device__ __forceinline__ void chord_epilogue(const double* a, const double* p,
                                               double gs, const double* sg,
                                               double c0, double* u, double* psi) {
  constexpr int NC = (WU ? NDIM : 0) + (WP ? 1 : 0);
  constexpr double INV2PI = 1.0 / (2.0 * kPI);
  constexpr double LN2_4PI = 0.69314718055994530942 / (4.0 * kPI);
  if (WU) {
    if (NDIM == 3) {
      u[0] = -INV2PI * (a[1] * p[2] - a[2] * p[1]);
      u[1] = -INV2PI * (a[2] * p[0] - a[0] * p[2]);
      u[2] = -INV2PI * (a[0] * p[1] - a[1] * p[0]);
    } else {
      u[0] = -INV2PI * a[1];
      u[1] = INV2PI * a[0];
    }
  }
  if (WP) {
    // the kernel dropped the skipped self pair (d = 0); remove its strength
    // from the sum of strengths
    double L = a[NC - 1];
    if (NDIM == 3) L -= (*sg - gs);
    *psi = -LN2_4PI * L;
  }
}

// Launch shapes.  FP32: 512-source tiles (32-byte duplicated records, 16 KB
// per buffer), target blocks of up to 1024; the default shape is 256 threads x
// 4 targets, and plan-time autotuning picks one of kF32Shapes.  FP64 (both
// forms): 128 threads x 2 targets, 256-source tiles (8 KB).
constexpr int F32_NT = 256, F32_R = 4, F32_TILE = 512;
constexpr int F32_TB = 1024;  // target padding: every FP32 shape divides it
constexpr int F64_NT = 128, F64_R = 2, F64_TILE = 256;

// FP32 kernel shapes: threads, targets per thread, minimum resident CTAs per
// SM (a register cap through __launch_bounds__).
struct F32Shape {
  int nt, r, minb;
};
constexpr int kNumF32Shapes = 6;
constexpr F32Shape kF32Shapes[kNumF32Shapes] = {
    {256, 4, 3},  // <= 85 registers: 24 warps / SM
    {256, 4, 4},  // <= 64 registers: 32 warps / SM
    {128, 8, 4},  // <= 128 registers: 16 warps, 8 targets per source load
    {256, 2, 5},  // <= 51 registers: 40 warps / SM
    {128, 8, 3},  // <= 170 registers: 12 warps, 8 targets per source load
    {256, 4, 2},  // <= 128 registers: 16 warps / SM
};

}  // namespace lpm

// ffmath.cuh -- device math of the octree far field: the order-4 Cartesian
// expansion of the chord-form sphere kernel about a cell centre, and the
// input features of the learned correction.
//
// Kernel (chord form; equals the reference biot_savart of
// src/lpm_sphere_functions.hpp:44-57 with 1 - x.y + eps^2 = q/2 for unit
// vectors):  u(x) = -(1/2pi) sum_j g_j (x cross y_j) / q_j,
//            q_j = |x - y_j|^2 + 2 eps^2.
// With d = x - c, y = c + delta, R^2 = |d|^2 + 2 eps^2:
//   1/q = (1/R^2) sum_n P_n(delta),  P_0 = 1, P_1 = 2 a.delta,
//   P_n = 2 (a.delta) P_(n-1) - s |delta|^2 P_(n-2),  a = d/R^2, s = 1/R^2
// (the generating function of the Chebyshev polynomials U_n).  Truncating at
// total order 4 in delta gives
//   u ~ -(1/2pi) x cross W,  W = (c S + V) / R^2,
//   S = sum_(n<=4) sum_j g_j P_n(delta_j),  V = sum_(n<=3) sum_j g_j delta_j P_n(delta_j),
// and both sums are contractions of the cell's moments to order 4 with
// powers of a.  The accumulated chord quantity is w = -W (velocity
// u = -(1/2pi) w cross x).
#pragma once

#include <cstdint>
#include <utility>

#include "farfield.hpp"

namespace lpm {
namespace ff {

// 35 monomials of degree <= 4, by degree then exponents descending
// (compile-time tables; sfor<N> unrolls a loop with a constant index).
__host__ __device__ constexpr int mono_exp(int i, int c) {
  int k = 0;
  for (int n = 0; n <= 4; ++n)
    for (int a = n; a >= 0; --a)
      for (int b = n - a; b >= 0; --b) {
        if (k == i) return c == 0 ? a : (c == 1 ? b : n - a - b);
        ++k;
      }
  return -1;
}
__host__ __device__ constexpr int mono_deg(int i) {
  return mono_exp(i, 0) + mono_exp(i, 1) + mono_exp(i, 2);
}
__host__ __device__ constexpr int mono_index(int a, int b, int c) {
  for (int i = 0; i < 35; ++i)
    if (mono_exp(i, 0) == a && mono_exp(i, 1) == b && mono_exp(i, 2) == c) return i;
  return -1;
}
// index of b + e_c
__host__ __device__ constexpr int mono_up(int i, int c) {
  return mono_index(mono_exp(i, 0) + (c == 0), mono_exp(i, 1) + (c == 1), mono_exp(i, 2) + (c == 2));
}
__host__ __device__ constexpr int fact(int n) { return n <= 1 ? 1 : n * fact(n - 1); }
// |b|! / (b1! b2! b3!)
__host__ __device__ constexpr float mono_mult(int i) {
  return float(fact(mono_deg(i)) /
               (fact(mono_exp(i, 0)) * fact(mono_exp(i, 1)) * fact(mono_exp(i, 2))));
}

template <class F, int... I>
__device__ __forceinline__ void sfor_impl(F& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// Complex moments from the real cell-frame moments: feature j (0..34) is the
// real or imaginary part of z^p conj(z)^q w^k summed over the points,
// z = d1 + i d2, w = d3, ordered by k, then n = p + q, then p descending
// (p >= q; p > q gives Re and Im, p = q only Re).  Expanding
// (u + i v)^p (u - i v)^q over powers of v gives each part as at most five
// real moments with integer coefficients; deg[j] = p + q + k.
struct CplxTable {
  int idx[35][5];
  float coef[35][5];
  int nterm[35];
  int deg[35];
};
constexpr CplxTable make_cplx_table() {
  CplxTable T{};
  int j = 0;
  for (int k = 0; k <= 4; ++k)
    for (int n = 0; n <= 4 - k; ++n)
      for (int p = n; 2 * p >= n; --p) {
        const int q = n - p;
        double cre[6] = {1, 0, 0, 0, 0, 0}, cim[6] = {0, 0, 0, 0, 0, 0};
        int deg = 0;
        for (int f = 0; f < p + q; ++f) {
          const double sg = f < p ? 1.0 : -1.0;  // times (u + sg i v)
          double nre[6] = {0, 0, 0, 0, 0, 0}, nim[6] = {0, 0, 0, 0, 0, 0};
          for (int b = 0; b <= deg; ++b) {
            nre[b] += cre[b];
            nim[b] += cim[b];
            nre[b + 1] += -sg * cim[b];
            nim[b + 1] += sg * cre[b];
          }
          ++deg;
          for (int b = 0; b <= deg; ++b) cre[b] = nre[b], cim[b] = nim[b];
        }
        for (int part = 0; part < (2 * p > n ? 2 : 1); ++part) {
          int m = 0;
          for (int b = 0; b <= n; ++b) {
            const double c = part == 0 ? cre[b] : cim[b];
            if (c != 0.0) {
              T.idx[j][m] = mono_index(n - b, b, k);
              T.coef[j][m] = float(c);
              ++m;
            }
          }
          T.nterm[j] = m;
          T.deg[j] = n + k;
          ++j;
        }
      }
  return T;
}

// Weighted powers A_b = mult_b a^b of a 3-vector.
__device__ __forceinline__ void weighted_powers(float a0, float a1, float a2, float* A) {
  float p0[5], p1[5], p2[5];
  p0[0] = p1[0] = p2[0] = 1.f;
#pragma unroll
  for (int k = 1; k <= 4; ++k) {
    p0[k] = p0[k - 1] * a0;
    p1[k] = p1[k - 1] * a1;
    p2[k] = p2[k - 1] * a2;
  }
  sfor<35>([&](auto I) {
    constexpr int i = decltype(I)::value;
    A[i] = mono_mult(i) * p0[mono_exp(i, 0)] * p1[mono_exp(i, 1)] * p2[mono_exp(i, 2)];
  });
}

// Order-4 expansion of one cell at cell-frame offset d = Q (x - c):
// returns W' (cell frame) with W = Q^T W'.  cell points at the record.
__device__ __forceinline__ void expand4(const float* cell, float d0, float d1, float d2, float c0,
                                        float* W) {
  const float R2 = d0 * d0 + d1 * d1 + d2 * d2 + c0;
  const float s = __fdividef(1.f, R2);  // ~2 ulp, far below the expansion's truncation error
  float A[35];
  weighted_powers(d0 * s, d1 * s, d2 * s, A);
  const float* M = cell + kCellM;
  const float* N1 = cell + kCellN1;
  float T[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  sfor<35>([&](auto I) {
    constexpr int i = decltype(I)::value;
    T[mono_deg(i)] = fmaf(A[i], M[i], T[mono_deg(i)]);
  });
  float T1[3] = {0.f, 0.f, 0.f};
  sfor<10>([&](auto I) {
    constexpr int i = decltype(I)::value;
    T1[mono_deg(i)] = fmaf(A[i], N1[i], T1[mono_deg(i)]);
  });
  const float T02 = cell[kCellN2];
  float U[4][3], U1[2][3];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int c = 0; c < 3; ++c) U[m][c] = 0.f;
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int c = 0; c < 3; ++c) U1[m][c] = 0.f;
  sfor<20>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int d = mono_deg(i);
    U[d][0] = fmaf(A[i], M[mono_up(i, 0)], U[d][0]);
    U[d][1] = fmaf(A[i], M[mono_up(i, 1)], U[d][1]);
    U[d][2] = fmaf(A[i], M[mono_up(i, 2)], U[d][2]);
  });
  sfor<4>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int d = mono_deg(i);
    U1[d][0] = fmaf(A[i], N1[mono_up(i, 0)], U1[d][0]);
    U1[d][1] = fmaf(A[i], N1[mono_up(i, 1)], U1[d][1]);
    U1[d][2] = fmaf(A[i], N1[mono_up(i, 2)], U1[d][2]);
  });
  const float S = T[0] + 2.f * T[1] + (4.f * T[2] - s * T1[0]) + (8.f * T[3] - 4.f * s * T1[1]) +
                  (16.f * T[4] - 12.f * s * T1[2] + s * s * T02);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float V = U[0][c] + 2.f * U[1][c] + (4.f * U[2][c] - s * U1[0][c]) +
                    (8.f * U[3][c] - 4.f * s * U1[1][c]);
    W[c] = V * s;
  }
  W[2] += cell[3] * S * s;  // centre (0, 0, |c|) in the cell frame
}

// Cell-frame offset of x from the cell.
__device__ __forceinline__ void to_cell(const float* cell, float x0, float x1, float x2, float* d) {
  const float e0 = x0 - cell[0], e1 = x1 - cell[1], e2 = x2 - cell[2];
#pragma unroll
  for (int r = 0; r < 3; ++r) d[r] = cell[8 + 3 * r] * e0 + cell[9 + 3 * r] * e1 + cell[10 + 3 * r] * e2;
}
__device__ __forceinline__ void from_cell(const float* cell, const float* v, float* out) {
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c] = cell[8 + c] * v[0] + cell[11 + c] * v[1] + cell[14 + c] * v[2];
}

// Learned-correction geometry of one (target, cell) pair.
struct PairGeo {
  float cs, sn;   // canonical rotation about the cell normal
  float D, rho;   // |x - c|, h / D
  float dt, dn;   // tangential and normal offset in the canonical frame
  float scale;    // S rho^5 / (2 pi D): normalisation of the residual
};

__device__ __forceinline__ PairGeo pair_geo(const float* cell, const float* d) {
  PairGeo g;
  const float t2 = d[0] * d[0] + d[1] * d[1];
  g.D = sqrtf(t2 + d[2] * d[2]);
  g.dt = sqrtf(t2);
  g.dn = d[2];
  if (g.dt > 0.f) {
    g.cs = d[0] / g.dt;
    g.sn = d[1] / g.dt;
  } else {
    g.cs = 1.f;
    g.sn = 0.f;
  }
  const float h = cell[4];
  g.rho = g.D > 0.f ? h / g.D : 1e30f;
  const float r2 = g.rho * g.rho;
  g.scale = g.D > 0.f ? cell[5] * r2 * r2 * g.rho / (6.283185307179586f * g.D) : 0.f;
  return g;
}

// Raw features (before normalisation), 41 values: 35 rotated complex
// moments, dt/D, dn/D, rho, eps/D, h; feature kBiasIn is set by the caller.
__device__ __forceinline__ void pair_features(const float* cell, const PairGeo& g, float eps,
                                              float* f) {
  // e^{i m phi}, m = 0..4
  float cm[5], sm[5];
  cm[0] = 1.f;
  sm[0] = 0.f;
#pragma unroll
  for (int m = 1; m <= 4; ++m) {
    cm[m] = cm[m - 1] * g.cs - sm[m - 1] * g.sn;
    sm[m] = sm[m - 1] * g.cs + cm[m - 1] * g.sn;
  }
  const float* C = cell + kCellC;
  int j = 0;
#pragma unroll
  for (int k = 0; k <= 4; ++k)
#pragma unroll
    for (int n = 0; n <= 4 - k; ++n)
#pragma unroll
      for (int p = n; 2 * p >= n; --p) {
        const int m = 2 * p - n;  // p - q
        if (m > 0) {
          const float re = C[j], im = C[j + 1];
          f[j] = re * cm[m] + im * sm[m];
          f[j + 1] = im * cm[m] - re * sm[m];
          j += 2;
        } else {
          f[j] = C[j];
          j += 1;
        }
      }
  const float iD = g.D > 0.f ? 1.f / g.D : 0.f;
  f[35] = g.dt * iD;
  f[36] = g.dn * iD;
  f[37] = g.rho;
  f[38] = eps * iD;
  f[39] = cell[4];
}

// Network output (canonical frame, normalised) -> chord-sum correction dw
// (global frame) at unit vector x: R = residual velocity, dw = 2 pi R x x.
__device__ __forceinline__ void correction(const float* cell, const PairGeo& g, const float* o,
                                           float oscale, float x0, float x1, float x2, float* dw) {
  const float k = oscale * g.scale;
  const float r0 = o[0] * k, r1 = o[1] * k, r2 = o[2] * k;
  const float v[3] = {r0 * g.cs - r1 * g.sn, r0 * g.sn + r1 * g.cs, r2};
  float R[3];
  from_cell(cell, v, R);
  const float tp = 6.283185307179586f;
  dw[0] = tp * (R[1] * x2 - R[2] * x1);
  dw[1] = tp * (R[2] * x0 - R[0] * x2);
  dw[2] = tp * (R[0] * x1 - R[1] * x0);
}

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// SiLU(z) = z sigma(z), sigma(z) = (1 + tanh(z/2)) / 2
__device__ __forceinline__ float silu(float z) {
  return 0.5f * z * (1.f + tanh_approx(0.5f * z));
}
__device__ __forceinline__ float silu_grad(float z) {
  const float sg = 0.5f * (1.f + tanh_approx(0.5f * z));
  return sg * (1.f + z * (1.f - sg));
}

}  // namespace ff
}  // namespace lpm

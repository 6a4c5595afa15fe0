// ics.cpp -- initial relative vorticity fields (host, FP64) for the
// direct-sum configurations.  Each follows a functor of
// src/lpm_vorticity_gallery.hpp; the Bessel functions are the rational
// Chebyshev-type approximations published in Numerical Recipes (Press et al.,
// 2nd ed., section 6.5, bessj0/bessj1), which is also what the reference uses
// (src/util/lpm_math.hpp:310-418).

#include <cmath>
#include <cstdint>
#include <stdexcept>

#include "lpm_gb300.h"
#include "lpm_host.hpp"

namespace lpm {
namespace {

constexpr double PI = 3.1415926535897932384626433832795;
constexpr double ZTOL = 2.220446049250313e-16;  // FloatingPoint<Real>::zero_tol

// Longitude in [0, 2 pi) (atan4, src/util/lpm_math.hpp:70-100).
double atan4(double y, double x) {
  if (std::fabs(x) < ZTOL) {
    if (y > 0.0) return 0.5 * PI;
    if (y < 0.0) return 1.5 * PI;
    return 0.0;
  }
  if (std::fabs(y) < ZTOL) return x > 0.0 ? 0.0 : (x < 0.0 ? PI : 0.0);
  const double th = std::atan2(std::fabs(y), std::fabs(x));
  if (x > 0.0 && y > 0.0) return th;
  if (x < 0.0 && y > 0.0) return PI - th;
  if (x < 0.0 && y < 0.0) return PI + th;
  return 2 * PI - th;
}

// J0 by a ratio of polynomials in x^2 for |x| < 8 and the Hankel asymptotic
// form otherwise (Numerical Recipes bessj0).
double bessel_j0(double x) {
  if (std::fabs(x) < ZTOL) return 1.0;
  const double ax = std::fabs(x);
  if (ax < 8.0) {
    const double y = x * x;
    const double num = 57568490574.0 + y * (-13362590354.0 + y * (651619640.7 + y * (-11214424.18 + y * (77392.33017 + y * (-184.9052456)))));
    const double den = 57568490411.0 + y * (1029532985.0 + y * (9494680.718 + y * (59272.64853 + y * (267.8532712 + y * 1.0))));
    return num / den;
  }
  const double z = 8.0 / ax, y = z * z, xx = ax - 0.785398164;
  const double p = 1.0 + y * (-0.1098628627e-2 + y * (0.2734510407e-4 + y * (-0.2073370639e-5 + y * 0.2093887211e-6)));
  const double q = -0.1562499995e-1 + y * (0.1430488765e-3 + y * (-0.6911147651e-5 + y * (0.7621095161e-6 - y * 0.934935152e-7)));
  return std::sqrt(0.636619772 / ax) * (std::cos(xx) * p - z * std::sin(xx) * q);
}

// J1 (Numerical Recipes bessj1).
double bessel_j1(double x) {
  const double ax = std::fabs(x);
  if (ax < 8.0) {
    const double y = x * x;
    const double num = x * (72362614232.0 + y * (-7895059235.0 + y * (242396853.1 + y * (-2972611.439 + y * (15704.48260 + y * (-30.16036606))))));
    const double den = 144725228442.0 + y * (2300535178.0 + y * (18583304.74 + y * (99447.43394 + y * (376.9991397 + y * 1.0))));
    return num / den;
  }
  const double z = 8.0 / ax, y = z * z, xx = ax - 2.356194491;
  const double p = 1.0 + y * (0.183105e-2 + y * (-0.3516396496e-4 + y * (0.2457520174e-5 + y * (-0.240337019e-6))));
  const double q = 0.04687499995 + y * (-0.2002690873e-3 + y * (0.8449199096e-5 + y * (-0.88228987e-6 + y * 0.105787412e-6)));
  const double r = std::sqrt(0.636619772 / ax) * (std::cos(xx) * p - z * std::sin(xx) * q);
  return x < 0.0 ? -r : r;
}

// lamb_dipole_vorticity (src/lpm_vorticity_gallery.hpp:192-206).
double lamb_dipole(double x, double y, double xc, double yc, double radius,
                   double strength) {
  const double K0 = 3.8317;
  const double r = std::sqrt((x - xc) * (x - xc) + (y - yc) * (y - yc));
  if (r < radius && !(std::fabs(r) < ZTOL)) {
    const double k = K0 / radius;
    const double sintheta = y / r;  // as in the reference: uses y, not y - yc
    const double denom = bessel_j0(K0);
    return -2 * strength * k * bessel_j1(k * r) * sintheta / denom;
  }
  return 0.0;
}

double gaussian(const double* p, double str, double b, double lon,
                double lat) {
  const double c[3] = {std::cos(lon) * std::cos(lat),
                       std::sin(lon) * std::cos(lat), std::sin(lat)};
  const double distsq = 1.0 - p[0] * c[0] - p[1] * c[1] - p[2] * c[2];
  return str * std::exp(-(b * b) * distsq);
}

}  // namespace

void ic_eval(int kind, const double* prm, int np, int ndim, int64_t n,
             const double* x, double* zeta) {
  auto need = [&](int k) {
    if (np < k) throw std::invalid_argument("ic_eval: too few parameters");
  };
  switch (kind) {
    case LPM_IC_SOLID_BODY:  // SolidBodyRotation (:31-57)
      if (ndim != 3) throw std::invalid_argument("solid body needs ndim 3");
      for (int64_t i = 0; i < n; ++i) zeta[i] = 2 * (2 * PI) * x[3 * i + 2];
      break;
    case LPM_IC_GAUSSIAN_SPHERE: {  // GaussianVortexSphere (:59-102)
      need(6);
      if (ndim != 3) throw std::invalid_argument("gaussian needs ndim 3");
      for (int64_t i = 0; i < n; ++i) {
        const double* p = x + 3 * i;
        zeta[i] = gaussian(p, prm[0], prm[1], prm[2], prm[3]) - prm[4] +
                  2 * prm[5] * p[2];
      }
      break;
    }
    case LPM_IC_RH54: {  // RossbyHaurwitz54 (:104-147)
      need(2);
      if (ndim != 3) throw std::invalid_argument("RH54 needs ndim 3");
      for (int64_t i = 0; i < n; ++i) {
        const double* p = x + 3 * i;
        const double z = p[2];
        const double lon = atan4(p[1], p[0]);
        const double p54 = z * ((z * z - 1) * (z * z - 1));
        zeta[i] = 2 * prm[0] * z + 30 * prm[1] * std::cos(4 * lon) * p54;
      }
      break;
    }
    case LPM_IC_DIPOLE_PAIR: {  // CollidingDipolePairPlane (:208-259)
      need(8);
      if (ndim != 2) throw std::invalid_argument("dipole pair needs ndim 2");
      for (int64_t i = 0; i < n; ++i) {
        const double px = x[2 * i], py = x[2 * i + 1];
        zeta[i] = lamb_dipole(px, py, prm[2], prm[3], prm[1], prm[0]) +
                  lamb_dipole(px, py, prm[6], prm[7], prm[5], prm[4]);
      }
      break;
    }
    case LPM_IC_MULTI_GAUSSIAN: {
      need(1);
      const int k = int(prm[0]);
      need(1 + 4 * k);
      if (ndim != 3) throw std::invalid_argument("multi gaussian needs ndim 3");
      for (int64_t i = 0; i < n; ++i) {
        double s = 0;
        for (int v = 0; v < k; ++v) {
          const double* q = prm + 1 + 4 * v;
          s += gaussian(x + 3 * i, q[0], q[1], q[2], q[3]);
        }
        zeta[i] = s;
      }
      break;
    }
    default:
      throw std::invalid_argument("unknown initial condition kind");
  }
}

}  // namespace lpm

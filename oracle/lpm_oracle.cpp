// lpm_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// FP64 CPU restatement of the LPM direct-summation Biot-Savart path, used by
// the test-suite, the smoke check and the CPU-baseline leg of the benchmark as
// the checker.  The product (the CUDA library under lpm_gb300/) never links,
// loads or calls this file.
//
// Parity status: the reference cannot be compiled here (it needs Kokkos,
// KokkosKernels, MPI, spdlog and Catch2, none of which are present), and the
// reference holds no golden vectors for this path.  This restatement is pinned
// instead by the reference's own known answers: the geometry test values
// (tests/lpm_geometry_tests.cpp:133-227), the solid-body-rotation velocity and
// stream-function checks of examples/bve_rotation.cpp:147-166, the
// Rossby-Haurwitz 5-4 analytic velocity (src/lpm_velocity_gallery.hpp:270-287),
// tangency u.x = 0 (src/lpm_sphere_functions.hpp:62-78) and the second-order
// time-convergence test of tests/lpm_ic2d_tests.cpp:165-188.  Those pin the
// algorithm (constants, signs, stepping) but not the reference's own
// round-off: parity with the reference is "partially pinned".
//
// Arithmetic order.  Every pair formula below follows the reference expression
// left to right so that, compiled with -ffp-contract=off, each pair term is the
// value the reference computes on the same inputs.  Sums over sources run
// sequentially in source order, which is what a Kokkos TeamThreadRange
// reduction produces on the OpenMP back end with team size 1
// (src/lpm_bve_sphere_kernels.hpp:118-127).  A Neumaier-compensated variant of
// every sum is available ("compensated" argument) as a higher-accuracy check.
//
// Layout: all coordinate and vector arrays are row-major (AoS) n x ndim.
// Masks are one byte per face, nonzero = divided (excluded) face.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double PI = 3.1415926535897932384626433832795;

// Sequential sum with optional Neumaier compensation.
struct Acc {
  double s = 0.0;
  double c = 0.0;
  bool comp = false;
  explicit Acc(bool compensated) : comp(compensated) {}
  inline void add(double v) {
    if (!comp) {
      s += v;
      return;
    }
    const double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) {
      c += (s - t) + v;
    } else {
      c += (v - t) + s;
    }
    s = t;
  }
  inline double value() const { return comp ? s + c : s; }
};

// SphereGeometry::dot / cross, src/lpm_geometry.hpp:370-386.
inline double sdot(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
inline void scross(double* c, const double* a, const double* b) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Sphere-kernel form.  0 = the reference's 1 - x.y; 1 = the chord form
// |x - y|^2 / 2, equal to 1 - x.y for unit vectors and free of its
// cancellation; it keeps evaluating the sphere kernel at RK stage positions,
// which leave the unit sphere.  The chord form is not the reference's
// arithmetic: it is the oracle for the LPM_FP64_CHORD / LPM_FP32C paths.
int g_chord = 0;

// 1 - x.y, or the chord form
inline double one_minus_dot(const double* x, const double* y) {
  if (!g_chord) return 1 - sdot(x, y);
  const double d0 = x[0] - y[0], d1 = x[1] - y[1], d2 = x[2] - y[2];
  return 0.5 * (d0 * d0 + d1 * d1 + d2 * d2);
}

// greens_fn, src/lpm_sphere_functions.hpp:21-29.
inline double greens_fn(const double* tgt, const double* src, double vort,
                        double area) {
  const double circ = -vort * area;
  return std::log(one_minus_dot(tgt, src)) * circ / (4 * PI);
}

// biot_savart, src/lpm_sphere_functions.hpp:44-57.
inline void biot_savart(double* u, const double* tgt, const double* src,
                        double vort, double area) {
  scross(u, tgt, src);
  const double strength = -vort * area / (4 * PI * one_minus_dot(src, tgt));
  for (int j = 0; j < 3; ++j) u[j] *= strength;
}

// Incompressible2DKernels<SphereGeometry>::kernel_vals,
// src/lpm_incompressible2d_kernels.hpp:35-47.
// want_psi = false skips the stream function's log (the velocity terms are
// the same either way; the reference always computes both).
inline void sphere_kernel_vals(double* r, const double* x, const double* y,
                               double eps, bool want_psi = true) {
  const double arg = one_minus_dot(x, y) + eps * eps;
  scross(r, x, y);
  for (int k = 0; k < 3; ++k) r[k] /= (-4 * PI * arg);
  r[3] = want_psi ? -std::log(arg) / (4 * PI) : 0.0;
}

// Incompressible2DKernels<PlaneGeometry>::kernel_vals,
// src/lpm_incompressible2d_kernels.hpp:72-84.
inline void plane_kernel_vals(double* r, const double* x, const double* y,
                              double eps, bool want_psi = true) {
  const double xmy[2] = {x[0] - y[0], x[1] - y[1]};
  const double arg = (xmy[0] * xmy[0] + xmy[1] * xmy[1]) + eps * eps;
  const double denom = 2 * PI * arg;
  r[0] = -xmy[1] / denom;
  r[1] = xmy[0] / denom;
  r[2] = want_psi ? -std::log(arg) / (4 * PI) : 0.0;
}

int g_threads = 0;

inline void set_threads() {
#ifdef _OPENMP
  if (g_threads > 0) omp_set_num_threads(g_threads);
#endif
}

// One BVE reduction over all face slots for one target (the body of
// StreamReduceDistinct/VelocityReduceDistinct and their collocated twins,
// src/lpm_bve_sphere_kernels.hpp:20-82, 218-274).  self < 0 means distinct.
inline void bve_target(double* psi, double* u, const double* x, long self,
                       const double* fx, const double* zeta,
                       const double* area, const unsigned char* mask, long nf,
                       bool comp) {
  if (psi) {
    Acc a(comp);
    for (long j = 0; j < nf; ++j) {
      double p = 0;
      if (!mask[j] && j != self) p = greens_fn(x, fx + 3 * j, zeta[j], area[j]);
      a.add(p);
    }
    *psi = a.value();
  }
  if (u) {
    Acc a0(comp), a1(comp), a2(comp);
    for (long j = 0; j < nf; ++j) {
      double v[3] = {0, 0, 0};
      if (!mask[j] && j != self) biot_savart(v, x, fx + 3 * j, zeta[j], area[j]);
      a0.add(v[0]);
      a1.add(v[1]);
      a2.add(v[2]);
    }
    u[0] = a0.value();
    u[1] = a1.value();
    u[2] = a2.value();
  }
}

// One Incompressible2DReducer reduction for one target,
// src/lpm_incompressible2d_kernels.hpp:92-136.  skip_self < 0: no skip.
inline void ic2d_target(int ndim, double* u, double* psi, const double* x,
                        long skip_self, const double* y, const double* zeta,
                        const double* area, const unsigned char* mask, long n,
                        double eps, bool comp) {
  Acc a[4] = {Acc(comp), Acc(comp), Acc(comp), Acc(comp)};
  const int nvals = ndim + 1;
  for (long j = 0; j < n; ++j) {
    if (skip_self >= 0 && j == skip_self) continue;
    if (mask[j]) continue;
    const double gamma = zeta[j] * area[j];
    double r[4];
    if (ndim == 3)
      sphere_kernel_vals(r, x, y + 3 * j, eps, psi != nullptr);
    else
      plane_kernel_vals(r, x, y + 2 * j, eps, psi != nullptr);
    for (int k = 0; k < nvals; ++k) a[k].add(r[k] * gamma);
  }
  if (u)
    for (int k = 0; k < ndim; ++k) u[k] = a[k].value();
  if (psi) *psi = a[ndim].value();
}

// KokkosBlas::scal(y, a, x): y = a*x  (KokkosKernels 4.7.00 BLAS-1, called at
// src/lpm_bve_rk4_impl.hpp:85-147).
inline void scal(double* y, double a, const double* x, long n) {
  for (long i = 0; i < n; ++i) y[i] = a * x[i];
}
// KokkosBlas::update(a, x, b, y, c, z): z = a*x + b*y + c*z; for c == 0 the
// old z is not read.
inline void update(double a, const double* x, double b, const double* y,
                   double c, double* z, long n) {
  if (c == 0.0) {
    for (long i = 0; i < n; ++i) z[i] = a * x[i] + b * y[i];
  } else {
    for (long i = 0; i < n; ++i) z[i] = a * x[i] + b * y[i] + c * z[i];
  }
}

}  // namespace

extern "C" {

int oracle_version(void) { return 1; }

void oracle_set_threads(int n) { g_threads = n; }

// 0: the reference's sphere arithmetic (default); 1: chord form.
void oracle_set_sphere_form(int chord) { g_chord = chord ? 1 : 0; }

int oracle_max_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

// BVEVertexSolve / BVEVertexStreamFn / BVEVertexVelocity
// (src/lpm_bve_sphere_kernels.hpp:90-211): psi and/or u at nv vertex targets
// from nf face slots.  psi or u may be null.  tgt_idx (optional) selects a
// subset of targets: output row k belongs to target tgt_idx[k].
void oracle_bve_vertex_solve(double* psi, double* u, const double* vx,
                             long nv, const long* tgt_idx, const double* fx,
                             const double* zeta, const double* area,
                             const unsigned char* mask, long nf,
                             int compensated) {
  set_threads();
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nv; ++k) {
    const long i = tgt_idx ? tgt_idx[k] : k;
    bve_target(psi ? psi + k : nullptr, u ? u + 3 * k : nullptr, vx + 3 * i,
               -1, fx, zeta, area, mask, nf, compensated != 0);
  }
}

// BVEFaceSolve / BVEFaceStreamFn / BVEFaceVelocity
// (src/lpm_bve_sphere_kernels.hpp:284-394): collocated, i != j skipped.
void oracle_bve_face_solve(double* psi, double* u, long nt,
                           const long* tgt_idx, const double* fx,
                           const double* zeta, const double* area,
                           const unsigned char* mask, long nf,
                           int compensated) {
  set_threads();
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const long i = tgt_idx ? tgt_idx[k] : k;
    bve_target(psi ? psi + k : nullptr, u ? u + 3 * k : nullptr, fx + 3 * i,
               i, fx, zeta, area, mask, nf, compensated != 0);
  }
}

// Incompressible2DPassiveSums (src/lpm_incompressible2d_kernels.hpp:144-193).
void oracle_ic2d_passive_sums(int ndim, double* u, double* psi,
                              const double* x, long nx, const long* tgt_idx,
                              const double* y, const double* zeta,
                              const double* area, const unsigned char* mask,
                              double eps, long n_active, int compensated) {
  set_threads();
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nx; ++k) {
    const long i = tgt_idx ? tgt_idx[k] : k;
    ic2d_target(ndim, u ? u + ndim * k : nullptr, psi ? psi + k : nullptr,
                x + ndim * i, -1, y, zeta, area, mask, n_active, eps,
                compensated != 0);
  }
}

// Incompressible2DActiveSums (src/lpm_incompressible2d_kernels.hpp:201-246).
// self_rule 0 = reference rule: skip i == j only when eps is zero
// (FloatingPoint<Real>::zero(eps), :235), so the self term is included for
// eps > 0; self_rule 1 = always skip i == j (the BVE collocated rule).
void oracle_ic2d_active_sums(int ndim, double* u, double* psi, long nt,
                             const long* tgt_idx, const double* y,
                             const double* zeta, const double* area,
                             const unsigned char* mask, double eps,
                             long n_active, int self_rule, int compensated) {
  set_threads();
  const bool eps_zero = std::fabs(eps) < 2.220446049250313e-16;
  const bool skip = (self_rule == 1) || eps_zero;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nt; ++k) {
    const long i = tgt_idx ? tgt_idx[k] : k;
    ic2d_target(ndim, u ? u + ndim * k : nullptr, psi ? psi + k : nullptr,
                y + ndim * i, skip ? i : -1, y, zeta, area, mask, n_active,
                eps, compensated != 0);
  }
}

// One sphere velocity evaluation used by the BVE stepper: eps == 0 uses the
// BVE functors (biot_savart); eps > 0 uses the smoothed sphere kernel of
// Incompressible2DKernels with the BVE rule that face targets skip i == j.
static void bve_velocity(double* vvel, const double* vx, long nv, double* fvel,
                         const double* fx, const double* fzeta,
                         const double* farea, const unsigned char* fmask,
                         long nf, double eps) {
  if (eps == 0.0) {
    oracle_bve_vertex_solve(nullptr, vvel, vx, nv, nullptr, fx, fzeta, farea,
                            fmask, nf, 0);
    oracle_bve_face_solve(nullptr, fvel, nf, nullptr, fx, fzeta, farea, fmask,
                          nf, 0);
  } else {
    oracle_ic2d_passive_sums(3, vvel, nullptr, vx, nv, nullptr, fx, fzeta,
                             farea, fmask, eps, nf, 0);
    oracle_ic2d_active_sums(3, fvel, nullptr, nf, nullptr, fx, fzeta, farea,
                            fmask, eps, nf, 1, 0);
  }
}

// BVEVorticityTendency (src/lpm_bve_sphere_kernels.hpp:399-413).
static void bve_tendency(double* dzeta, const double* vel, long n, double dt,
                         double Omega) {
  for (long i = 0; i < n; ++i) dzeta[i] = -2.0 * Omega * vel[3 * i + 2] * dt;
}

// BVERK4::advance_timestep (src/lpm_bve_rk4_impl.hpp:63-167) with the update
// functor BVERK4Update (:12-53).  fix_facevort3 = 0 reproduces the reference,
// whose face update passes facevort4 in place of facevort3 (:155-157).
// reproject != 0 renormalises positions to the unit sphere after the update
// (the reference does not).  vvel/fvel hold the velocities of the current
// state on entry and of the new state on exit.
void oracle_bve_rk4_step(long nv, double* vx, double* vzeta, double* vvel,
                         long nf, double* fx, double* fzeta, double* fvel,
                         const double* farea, const unsigned char* fmask,
                         double dt, double Omega, double eps,
                         int fix_facevort3, int reproject) {
  std::vector<double> vx1(3 * nv), vx2(3 * nv), vx3(3 * nv), vx4(3 * nv),
      vxw(3 * nv);
  std::vector<double> vz1(nv), vz2(nv), vz3(nv), vz4(nv), vzw(nv);
  std::vector<double> fx1(3 * nf), fx2(3 * nf), fx3(3 * nf), fx4(3 * nf),
      fxw(3 * nf);
  std::vector<double> fz1(nf), fz2(nf), fz3(nf), fz4(nf), fzw(nf);

  // stage 1
  scal(vx1.data(), dt, vvel, 3 * nv);
  bve_tendency(vz1.data(), vvel, nv, dt, Omega);
  scal(fx1.data(), dt, fvel, 3 * nf);
  bve_tendency(fz1.data(), fvel, nf, dt, Omega);

  double* vxs[3] = {vx1.data(), vx2.data(), vx3.data()};
  double* vzs[3] = {vz1.data(), vz2.data(), vz3.data()};
  double* fxs[3] = {fx1.data(), fx2.data(), fx3.data()};
  double* fzs[3] = {fz1.data(), fz2.data(), fz3.data()};
  double* vxo[3] = {vx2.data(), vx3.data(), vx4.data()};
  double* vzo[3] = {vz2.data(), vz3.data(), vz4.data()};
  double* fxo[3] = {fx2.data(), fx3.data(), fx4.data()};
  double* fzo[3] = {fz2.data(), fz3.data(), fz4.data()};
  const double coef[3] = {0.5, 0.5, 1.0};
  for (int s = 0; s < 3; ++s) {
    update(1.0, vx, coef[s], vxs[s], 0.0, vxw.data(), 3 * nv);
    update(1.0, vzeta, coef[s], vzs[s], 0.0, vzw.data(), nv);
    update(1.0, fx, coef[s], fxs[s], 0.0, fxw.data(), 3 * nf);
    update(1.0, fzeta, coef[s], fzs[s], 0.0, fzw.data(), nf);
    bve_velocity(vvel, vxw.data(), nv, fvel, fxw.data(), fzw.data(), farea,
                 fmask, nf, eps);
    scal(vxo[s], dt, vvel, 3 * nv);
    scal(fxo[s], dt, fvel, 3 * nf);
    bve_tendency(vzo[s], vvel, nv, dt, Omega);
    bve_tendency(fzo[s], fvel, nf, dt, Omega);
  }
  const double sixth = 1.0 / 6.0;
  const double third = 1.0 / 3.0;
  for (long i = 0; i < nv; ++i) {
    for (int j = 0; j < 3; ++j) {
      const long k = 3 * i + j;
      vx[k] += sixth * (vx1[k] + vx4[k]) + third * (vx2[k] + vx3[k]);
    }
    vzeta[i] += sixth * (vz1[i] + vz4[i]) + third * (vz2[i] + vz3[i]);
  }
  const double* fz3u = fix_facevort3 ? fz3.data() : fz4.data();
  for (long i = 0; i < nf; ++i) {
    for (int j = 0; j < 3; ++j) {
      const long k = 3 * i + j;
      fx[k] += sixth * (fx1[k] + fx4[k]) + third * (fx2[k] + fx3[k]);
    }
    fzeta[i] += sixth * (fz1[i] + fz4[i]) + third * (fz2[i] + fz3u[i]);
  }
  if (reproject) {
    for (long i = 0; i < nv; ++i) {
      double* p = vx + 3 * i;
      const double r = std::sqrt(sdot(p, p));
      for (int j = 0; j < 3; ++j) p[j] /= r;
    }
    for (long i = 0; i < nf; ++i) {
      double* p = fx + 3 * i;
      const double r = std::sqrt(sdot(p, p));
      for (int j = 0; j < 3; ++j) p[j] /= r;
    }
  }
  bve_velocity(vvel, vx, nv, fvel, fx, fzeta, farea, fmask, nf, eps);
}

// Incompressible2DTendencies (src/lpm_incompressible2d_kernels.hpp:257-278)
// with CoriolisSphere::dfdt = 2*Omega*u[2] (src/lpm_coriolis.hpp:181-184) or
// CoriolisBetaPlane::dfdt = beta*u[1] (:139-142).
static void ic2d_tendency(int ndim, double* dzeta, const double* u, long n,
                          double cor) {
  for (long i = 0; i < n; ++i) {
    dzeta[i] = (ndim == 3) ? -(2 * cor * u[3 * i + 2]) : -(cor * u[2 * i + 1]);
  }
}

static void ic2d_sums(int ndim, double* vvel, double* vpsi, const double* vx,
                      long nv, double* fvel, double* fpsi, const double* fx,
                      const double* fzeta, const double* farea,
                      const unsigned char* fmask, long nf, double eps,
                      int self_rule) {
  oracle_ic2d_passive_sums(ndim, vvel, vpsi, vx, nv, nullptr, fx, fzeta, farea,
                           fmask, eps, nf, 0);
  oracle_ic2d_active_sums(ndim, fvel, fpsi, nf, nullptr, fx, fzeta, farea,
                          fmask, eps, nf, self_rule, 0);
}

// Incompressible2D::init_direct_sums (src/lpm_incompressible2d_impl.hpp:235-254).
void oracle_ic2d_init_direct_sums(int ndim, long nv, const double* vx,
                                  double* vvel, double* vpsi, long nf,
                                  const double* fx, const double* fzeta,
                                  double* fvel, double* fpsi,
                                  const double* farea,
                                  const unsigned char* fmask, double eps,
                                  int self_rule) {
  ic2d_sums(ndim, vvel, vpsi, vx, nv, fvel, fpsi, fx, fzeta, farea, fmask, nf,
            eps, self_rule);
}

// Incompressible2DRK2::advance_timestep_impl
// (src/lpm_incompressible2d_rk2_impl.hpp:74-172).  cor = Omega (sphere) or
// beta (plane).  vvel/fvel/vpsi/fpsi hold the current state's sums on entry.
void oracle_ic2d_rk2_step(int ndim, long nv, double* vx, double* vzeta,
                          double* vvel, double* vpsi, long nf, double* fx,
                          double* fzeta, double* fvel, double* fpsi,
                          const double* farea, const unsigned char* fmask,
                          double dt, double eps, double cor, int self_rule) {
  const long dv = ndim * nv, df = ndim * nf;
  std::vector<double> vx1(dv), vx2(dv), vxw(dv), vz1(nv), vz2(nv), vzw(nv);
  std::vector<double> fx1(df), fx2(df), fxw(df), fz1(nf), fz2(nf), fzw(nf);
  scal(vx1.data(), dt, vvel, dv);
  scal(fx1.data(), dt, fvel, df);
  ic2d_tendency(ndim, vz1.data(), vvel, nv, cor);
  ic2d_tendency(ndim, fz1.data(), fvel, nf, cor);
  update(1, vzeta, dt, vz1.data(), 0, vzw.data(), nv);
  update(1, fzeta, dt, fz1.data(), 0, fzw.data(), nf);
  update(1, vx, dt, vvel, 0, vxw.data(), dv);
  update(1, fx, dt, fvel, 0, fxw.data(), df);
  ic2d_sums(ndim, vvel, vpsi, vxw.data(), nv, fvel, fpsi, fxw.data(),
            fzw.data(), farea, fmask, nf, eps, self_rule);
  scal(vx2.data(), dt, vvel, dv);
  scal(fx2.data(), dt, fvel, df);
  ic2d_tendency(ndim, vz2.data(), vvel, nv, cor);
  ic2d_tendency(ndim, fz2.data(), fvel, nf, cor);
  update(0.5 * dt, vz1.data(), 0.5 * dt, vz2.data(), 1, vzeta, nv);
  update(0.5 * dt, fz1.data(), 0.5 * dt, fz2.data(), 1, fzeta, nf);
  update(0.5, vx1.data(), 0.5, vx2.data(), 1, vx, dv);
  update(0.5, fx1.data(), 0.5, fx2.data(), 1, fx, df);
  ic2d_sums(ndim, vvel, vpsi, vx, nv, fvel, fpsi, fx, fzeta, farea, fmask, nf,
            eps, self_rule);
}

// Incompressible2D::total_vorticity / total_enstrophy / total_kinetic_energy
// (src/lpm_incompressible2d_impl.hpp:91-137), sequential order.
void oracle_invariants(int ndim, long nf, const double* zeta,
                       const double* vel, const double* area,
                       const unsigned char* mask, double* out3) {
  double tv = 0, te = 0, tk = 0;
  for (long i = 0; i < nf; ++i) {
    tv += (mask[i] ? 0 : zeta[i] * area[i]);
    te += (mask[i] ? 0 : (zeta[i] * zeta[i]) * area[i]);
    if (!mask[i]) {
      double n2 = 0;
      for (int k = 0; k < ndim; ++k) n2 += vel[ndim * i + k] * vel[ndim * i + k];
      tk += n2 * area[i];
    }
  }
  out3[0] = tv;
  out3[1] = 0.5 * te;
  out3[2] = 0.5 * tk;
}

// ErrNorms (src/lpm_error.hpp:81-91, src/lpm_error_impl.hpp:58-85,155-162):
// l1, l2 weighted by wt, linf = max|err| / max|exact|, on vector magnitudes
// (ndim > 1) or absolute values (ndim == 1).  wt may be null (weight 1).
// mask (optional) excludes entries, like the masked constructor.
void oracle_err_norms(int ndim, long n, const double* appx,
                      const double* exact, const double* wt,
                      const unsigned char* mask, double* out3) {
  double l1n = 0, l1d = 0, l2n = 0, l2d = 0, lin = 0, lid = 0;
  for (long i = 0; i < n; ++i) {
    if (mask && mask[i]) continue;
    double e2 = 0, x2 = 0;
    for (int k = 0; k < ndim; ++k) {
      const double e = appx[ndim * i + k] - exact[ndim * i + k];
      e2 += e * e;
      x2 += exact[ndim * i + k] * exact[ndim * i + k];
    }
    const double em = std::sqrt(e2), xm = std::sqrt(x2);
    const double w = wt ? wt[i] : 1.0;
    l1n += em * w;
    l1d += xm * w;
    l2n += em * em * w;
    l2d += xm * xm * w;
    if (em > lin) lin = em;
    if (xm > lid) lid = xm;
  }
  const double tol = 2.220446049250313e-16;
  auto safe = [tol](double x) { return x / (x * x + tol * tol); };
  out3[0] = l1n * safe(l1d);
  out3[1] = std::sqrt(l2n * safe(l2d));
  out3[2] = lin * safe(lid);
}

// Planar SWE direct sums with PSE (PlanarSWEVertexSums / PlanarSWEFaceSums,
// src/lpm_swe_kernels.hpp:626-876; pair term planar_swe_sums_rhs_pse :394-480,
// reducer rules :559-570; PSE kernel pse::BivariateOrder8::laplacian,
// src/lpm_pse.hpp:66-72, kernel_input = distance / pse_eps :30-34).
// out9[9 * i + k]: u, v, du/dx, du/dy, dv/dx, dv/dy, lap(s), psi, phi.
// collocated: targets are the sources (face sums); then j == i is skipped.
void oracle_swe_plane_sums(long nt, const double* tx, const double* ts, long ns,
                           const double* y, const double* zeta, const double* sigma,
                           const double* area, const unsigned char* mask,
                           const double* ss, double eps, double pse_eps,
                           int collocated, double* out9) {
  const double epssq = eps * eps;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long i = 0; i < nt; ++i) {
    double r[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double x0 = tx[2 * i], x1 = tx[2 * i + 1];
    for (long j = 0; j < ns; ++j) {
      if (mask[j] || (collocated && i == j)) continue;
      const double d0 = x0 - y[2 * j], d1 = x1 - y[2 * j + 1];
      const double rsq = d0 * d0 + d1 * d1;
      const double denom = 2 * PI * (rsq + epssq);
      const double denom2 = PI * ((rsq + epssq) * (rsq + epssq));
      const double rot = zeta[j] * area[j];
      const double pot = sigma[j] * area[j];
      const double greens = -std::log(rsq + epssq) / (4 * PI);
      const double xy = d0 * d1;
      r[0] += (-d1 * rot + d0 * pot) / denom;
      r[1] += (d0 * rot + d1 * pot) / denom;
      r[2] += (xy * rot - (d0 * d0) * pot) / denom2 + pot / denom;
      r[3] += ((d1 * d1) * rot - xy * pot) / denom2 - rot / denom;
      r[4] += (-(d0 * d0) * rot - xy * pot) / denom2 + rot / denom;
      r[5] += (-xy * rot - (d1 * d1) * pot) / denom2 + pot / denom;
      // PSE: r = |y - x| / pse_eps
      const double e0 = y[2 * j] - x0, e1 = y[2 * j + 1] - x1;
      const double pr = std::sqrt(e0 * e0 + e1 * e1) / pse_eps;
      const double prsq = pr * pr;
      const double lap = (40 * (1 - prsq) + 10 * (prsq * prsq) - 2 * prsq * (prsq * prsq) / 3) *
                         (std::exp(-prsq) / PI);
      r[6] += (ss[j] - ts[i]) * area[j] * lap / (pse_eps * pse_eps);
      r[7] += greens * rot;
      r[8] += greens * pot;
    }
    for (int k = 0; k < 9; ++k) out9[9 * i + k] = r[k];
  }
}

// Spherical SWE direct sums (SphereVertexSums / SphereFaceSums,
// src/lpm_swe_kernels.hpp:723-940; pair term sphere_swe_velocity_sums
// :335-373, reducer rules SphereSweDirectSumReducer :608-619).
//
// Pair term, with s = x.y, D = (1 - s) + eps^2, c = x cross y,
// rot = -zeta A, pot = -sigma A:
//   velocity (kzeta_sphere + ksigma_sphere, :63-108)
//     u += c rot / (4 pi D) + (I - x x^T) y pot / (4 pi D)
//   gradient (grad_kzeta, grad_ksigma, :114-325) -- the reference writes each
//   entry as an expanded polynomial over 4 pi D^2; those polynomials equal
//     gkz = (D [y]x + c ((1 + eps^2) x - y)^T) / (4 pi D^2)      (identically)
//     gks = (w w^T - D (x w^T + s P)) / (4 pi D^2),  w = P y,  P = I - x x^T
//   (on the unit sphere), i.e. gkz = -(dK_zeta/dx) P and gks = +(dK_sigma/dx) P
//   for the kernels K_zeta = c / (4 pi D), K_sigma = P y / (4 pi D);
//     M += gkz rot + gks pot  (9 entries, row-major).
// The compact forms are used here; tests pin them against the reference's
// polynomials evaluated in extended precision (tests/golden/).
// Sums run in source order; masked sources are skipped, and with collocated
// targets (face sums with |eps| < DBL_EPSILON) so is j == i.  The velocity
// part follows the reference's operation order (velz + vels per pair); the
// reference leaves the 3-vectors velz and vels of :341-346 uninitialised
// before kzeta_sphere/ksigma_sphere add into them -- taken here as zero.
// out12[12 i + k]: u, v, w, then M (du/dx, du/dy, du/dz, dv/dx, ...).
void oracle_swe_sphere_sums(long nt, const double* tx, long ns, const double* y,
                            const double* zeta, const double* sigma, const double* area,
                            const unsigned char* mask, double eps, int collocated,
                            double* out12) {
  const double epssq = eps * eps;
  const double e1 = 1 + epssq;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long i = 0; i < nt; ++i) {
    const double* x = tx + 3 * i;
    double P[9];
    for (int a = 0; a < 3; ++a) {
      for (int b = 0; b < 3; ++b) P[3 * a + b] = -x[a] * x[b];
      P[4 * a] += 1;
    }
    double r[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (long j = 0; j < ns; ++j) {
      if (mask[j] || (collocated && i == j)) continue;
      const double* yj = y + 3 * j;
      const double s = sdot(x, yj);
      const double D = 1 - s + epssq;
      const double den1 = 4 * PI * D;
      const double rot = -zeta[j] * area[j];
      const double pot = -sigma[j] * area[j];
      const double sz = rot / den1, ss = pot / den1;
      double c[3];
      scross(c, x, yj);
      for (int a = 0; a < 3; ++a) {
        double w = 0;
        for (int b = 0; b < 3; ++b) w += P[3 * a + b] * yj[b];
        r[a] += c[a] * sz + w * ss;
      }
      const double den2 = 1.0 / (4 * PI * ((1 - s + epssq) * (1 - s + epssq)));
      const double Yx[9] = {0, -yj[2], yj[1], yj[2], 0, -yj[0], -yj[1], yj[0], 0};
      double v[3], w[3];
      for (int a = 0; a < 3; ++a) {
        v[a] = e1 * x[a] - yj[a];
        w[a] = yj[a] - s * x[a];
      }
      for (int a = 0; a < 3; ++a) {
        for (int b = 0; b < 3; ++b) {
          const double gkz = (D * Yx[3 * a + b] + c[a] * v[b]) * den2;
          const double gks = (w[a] * w[b] - D * (x[a] * w[b] + s * P[3 * a + b])) * den2;
          r[3 + 3 * a + b] += gkz * rot + gks * pot;
        }
      }
    }
    for (int k = 0; k < 12; ++k) out12[12 * i + k] = r[k];
  }
}

}  // extern "C"

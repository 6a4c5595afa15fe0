// lpm_gb300.hpp -- header-only C++17 facade over the C ABI (lpm_gb300.h) with
// the reference's class and method names.
//
// A reference build swaps its Kokkos functor launches for these calls, one
// call per launch site.  The facade needs no Kokkos: any view type with .data()
// and .stride(0)/.stride(1) (Kokkos::View<Real*[3]> in either layout, or the
// small DeviceArray below) converts to an lpm_view.  Nonzero status codes
// become std::runtime_error, as LPM_REQUIRE does (src/lpm_assert.hpp:22-30).
#ifndef LPM_GB300_HPP
#define LPM_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>

#include "lpm_gb300.h"

namespace lpm_gb300 {

inline void require(int rc, const char* what) {
  if (rc != LPM_OK)
    throw std::runtime_error(std::string(what) + ": " + lpm_last_error() +
                             " (status " + std::to_string(rc) + ")");
}

// Strided view of an n x ndim array from any view-like object.
template <typename V>
lpm_view as_view(const V& v) {
  return lpm_view{const_cast<double*>(reinterpret_cast<const double*>(v.data())),
                  static_cast<int64_t>(v.stride(0)), static_cast<int64_t>(v.stride(1))};
}
inline lpm_view as_view(double* p, int64_t stride_i, int64_t stride_c) {
  return lpm_view{p, stride_i, stride_c};
}

// Owns an lpm_context (device binding, stream, cached scratch).
class Context {
 public:
  explicit Context(int device = 0, int precision = LPM_FP64) {
    require(lpm_context_create(&h_, device), "lpm_context_create");
    require(lpm_context_set_precision(h_, precision), "lpm_context_set_precision");
  }
  ~Context() { lpm_context_destroy(h_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  lpm_context* get() const { return h_; }
  void set_stream(void* s) { require(lpm_context_set_stream(h_, s), "set_stream"); }
  void set_precision(int p) { require(lpm_context_set_precision(h_, p), "set_precision"); }
  void synchronize() { require(lpm_context_synchronize(h_), "synchronize"); }

 private:
  lpm_context* h_ = nullptr;
};

// ---- functor-equivalent calls (src/lpm_bve_sphere_kernels.hpp) ------------
inline void BVEVertexVelocity(Context& c, lpm_view u, lpm_view vx, int64_t nv, lpm_view fx,
                              const double* zeta, const double* area,
                              const uint8_t* mask, int64_t nf) {
  require(lpm_bve_vertex_velocity(c.get(), u, vx, nv, fx, zeta, area, mask, nf),
          "BVEVertexVelocity");
}
inline void BVEFaceVelocity(Context& c, lpm_view u, lpm_view fx, const double* zeta,
                            const double* area, const uint8_t* mask, int64_t nf) {
  require(lpm_bve_face_velocity(c.get(), u, fx, zeta, area, mask, nf), "BVEFaceVelocity");
}
inline void BVEVertexStreamFn(Context& c, double* psi, lpm_view vx, int64_t nv, lpm_view fx,
                              const double* zeta, const double* area,
                              const uint8_t* mask, int64_t nf) {
  require(lpm_bve_vertex_stream_fn(c.get(), psi, vx, nv, fx, zeta, area, mask, nf),
          "BVEVertexStreamFn");
}
inline void BVEFaceStreamFn(Context& c, double* psi, lpm_view fx, const double* zeta,
                            const double* area, const uint8_t* mask, int64_t nf) {
  require(lpm_bve_face_stream_fn(c.get(), psi, fx, zeta, area, mask, nf), "BVEFaceStreamFn");
}

// ---- shallow-water sums (src/lpm_swe_kernels.hpp) --------------------------
// PlanarSWEVertexSums / PlanarSWEFaceSums (:626-876)
inline void PlanarSWEVertexSums(Context& c, lpm_view u, double* ddot, double* du1dx1,
                                double* du1dx2, double* du2dx1, double* du2dx2, double* laps,
                                double* psi, double* phi, lpm_view vx, const double* vs,
                                int64_t nv, lpm_view fx, const double* zeta,
                                const double* sigma, const double* area, const uint8_t* mask,
                                const double* fs, int64_t nf, double eps, double pse_eps,
                                bool do_velocity) {
  require(lpm_swe_plane_vertex_sums(c.get(), u, ddot, du1dx1, du1dx2, du2dx1, du2dx2, laps, psi,
                                    phi, vx, vs, nv, fx, zeta, sigma, area, mask, fs, nf, eps,
                                    pse_eps, do_velocity ? 1 : 0),
          "PlanarSWEVertexSums");
}
inline void PlanarSWEFaceSums(Context& c, lpm_view u, double* ddot, double* du1dx1,
                              double* du1dx2, double* du2dx1, double* du2dx2, double* laps,
                              double* psi, double* phi, lpm_view fx, const double* zeta,
                              const double* sigma, const double* area, const uint8_t* mask,
                              const double* fs, int64_t nf, double eps, double pse_eps,
                              bool do_velocity) {
  require(lpm_swe_plane_face_sums(c.get(), u, ddot, du1dx1, du1dx2, du2dx1, du2dx2, laps, psi,
                                  phi, fx, zeta, sigma, area, mask, fs, nf, eps, pse_eps,
                                  do_velocity ? 1 : 0),
          "PlanarSWEFaceSums");
}
// SphereVertexSums / SphereFaceSums (:723-940); grad may be null
inline void SphereVertexSums(Context& c, lpm_view u, double* ddot, lpm_view vx, int64_t nv,
                             lpm_view fx, const double* zeta, const double* sigma,
                             const double* area, const uint8_t* mask, double eps, int64_t nf,
                             bool do_velocity, double* grad = nullptr) {
  require(lpm_swe_sphere_vertex_sums(c.get(), u, ddot, grad, vx, nv, fx, zeta, sigma, area, mask,
                                     nf, eps, do_velocity ? 1 : 0),
          "SphereVertexSums");
}
inline void SphereFaceSums(Context& c, lpm_view u, double* ddot, lpm_view fx, const double* zeta,
                           const double* sigma, const double* area, const uint8_t* mask,
                           double eps, int64_t nf, bool do_velocity, double* grad = nullptr) {
  require(lpm_swe_sphere_face_sums(c.get(), u, ddot, grad, fx, zeta, sigma, area, mask, nf, eps,
                                   do_velocity ? 1 : 0),
          "SphereFaceSums");
}

// ---- BVERK4 (src/lpm_bve_rk4.hpp:10-77) ----------------------------------
class BVERK4 {
 public:
  BVERK4(Context& c, double dt, int64_t nverts, int64_t nfaces, double Omega,
         double eps = 0.0, int precision = LPM_FP64, uint32_t flags = 0)
      : dt(dt), Omega(Omega) {
    require(lpm_bve_rk4_create(c.get(), &h_, nverts, nfaces, dt, Omega, eps, precision, flags),
            "BVERK4");
  }
  ~BVERK4() { lpm_bve_rk4_destroy(h_); }
  BVERK4(const BVERK4&) = delete;
  BVERK4& operator=(const BVERK4&) = delete;
  void advance_timestep(lpm_view vx, double* vzeta, lpm_view vvel, lpm_view fx, double* fzeta,
                        lpm_view fvel, const double* farea, const uint8_t* fmask) {
    require(lpm_bve_rk4_advance_timestep(h_, vx, vzeta, vvel, fx, fzeta, fvel, farea, fmask),
            "BVERK4::advance_timestep");
  }
  // evaluate the stages with an octree far field (LPM_FP64_CHORD steppers)
  void set_farfield(lpm_farfield* ff, int rebuild_every = 0) {
    require(lpm_bve_rk4_set_farfield(h_, ff, rebuild_every), "BVERK4::set_farfield");
  }
  double dt, Omega;

 private:
  lpm_bve_rk4* h_ = nullptr;
};

// Octree far field with the learned correction (no reference counterpart).
class FarField {
 public:
  explicit FarField(Context& c, double theta = 0.5, int leaf_max = 64, double rho_min = 0.25) {
    require(lpm_farfield_create(c.get(), &h_, theta, leaf_max, rho_min), "FarField");
  }
  ~FarField() { lpm_farfield_destroy(h_); }
  FarField(const FarField&) = delete;
  FarField& operator=(const FarField&) = delete;
  // trains on the GPU; loss (optional) receives one value per epoch
  void train(int64_t nsamples, int epochs, int batch, double lr, uint64_t seed, int level_min,
             int level_max, double eps, float* loss = nullptr) {
    require(lpm_farfield_train(h_, nsamples, epochs, batch, lr, seed, level_min, level_max, eps,
                               loss),
            "FarField::train");
  }
  void load(const float* w, const float* norm) {
    require(lpm_farfield_set_weights(h_, w, norm), "FarField::load");
  }
  void save(float* w, float* norm) { require(lpm_farfield_get_weights(h_, w, norm), "FarField::save"); }
  void set_network(bool on) { require(lpm_farfield_set_network(h_, on ? 1 : 0), "FarField::set_network"); }
  void velocity(lpm_view u, lpm_view x, int64_t nx, lpm_view fx, const double* zeta,
                const double* area, const uint8_t* mask, int64_t nf, double eps) {
    require(lpm_farfield_velocity(h_, u, x, nx, fx, zeta, area, mask, nf, eps),
            "FarField::velocity");
  }
  lpm_farfield* get() { return h_; }

 private:
  lpm_farfield* h_ = nullptr;
};

// Many independent BVE problems advanced together (one persistent launch per
// evaluation, graph-captured steps).
class BVEEnsemble {
 public:
  BVEEnsemble(Context& c, int nproblems, const int64_t* nverts, const int64_t* nfaces,
              const uint8_t* fmask, double dt, double Omega, double eps,
              int precision = LPM_FP32C, uint32_t flags = 0) {
    require(lpm_ensemble_create(c.get(), &h_, nproblems, nverts, nfaces, fmask, dt, Omega, eps,
                                precision, flags),
            "BVEEnsemble");
  }
  ~BVEEnsemble() { lpm_ensemble_destroy(h_); }
  BVEEnsemble(const BVEEnsemble&) = delete;
  BVEEnsemble& operator=(const BVEEnsemble&) = delete;
  void velocity(lpm_view vx, lpm_view vvel, lpm_view fx, const double* fzeta, lpm_view fvel,
                const double* farea) {
    require(lpm_ensemble_velocity(h_, vx, vvel, fx, fzeta, fvel, farea), "BVEEnsemble::velocity");
  }
  void advance_timestep(lpm_view vx, double* vzeta, lpm_view vvel, lpm_view fx, double* fzeta,
                        lpm_view fvel, const double* farea) {
    require(lpm_ensemble_advance_timestep(h_, vx, vzeta, vvel, fx, fzeta, fvel, farea),
            "BVEEnsemble::advance_timestep");
  }

 private:
  lpm_ensemble* h_ = nullptr;
};

// ---- Incompressible2DRK2 (src/lpm_incompressible2d_rk2.hpp) --------------
class Incompressible2DRK2 {
 public:
  Incompressible2DRK2(Context& c, int ndim, double dt, int64_t n_passive, int64_t n_active,
                      double eps, double coriolis, int precision = LPM_FP64,
                      uint32_t flags = 0)
      : dt(dt), eps(eps) {
    require(lpm_ic2d_rk2_create(c.get(), &h_, ndim, n_passive, n_active, dt, eps, coriolis,
                                precision, flags),
            "Incompressible2DRK2");
  }
  ~Incompressible2DRK2() { lpm_ic2d_rk2_destroy(h_); }
  Incompressible2DRK2(const Incompressible2DRK2&) = delete;
  Incompressible2DRK2& operator=(const Incompressible2DRK2&) = delete;
  void advance_timestep_impl(lpm_view vx, double* vzeta, lpm_view vvel, double* vpsi,
                             lpm_view fx, double* fzeta, lpm_view fvel, double* fpsi,
                             const double* farea, const uint8_t* fmask) {
    require(lpm_ic2d_rk2_advance_timestep(h_, vx, vzeta, vvel, vpsi, fx, fzeta, fvel, fpsi,
                                          farea, fmask),
            "Incompressible2DRK2::advance_timestep_impl");
    ++t_idx;
  }
  double dt, eps;
  int t_idx = 0;

 private:
  lpm_ic2d_rk2* h_ = nullptr;
};

}  // namespace lpm_gb300

#endif  // LPM_GB300_HPP

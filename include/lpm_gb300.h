/* lpm_gb300.h -- C ABI of the GB300 (sm_103a) direct-summation Biot-Savart
 * library.
 *
 * This is the drop-in boundary for LPM's direct-sum hot path.  Each entry point
 * replaces one Kokkos launch of the reference,
 *
 *     Kokkos::parallel_for(label, TeamPolicy<>(n_targets, AUTO()), Functor(...));
 *
 * with the same arguments in plain pointers and sizes, or one stepper method
 * (BVERK4::advance_timestep, Incompressible2DRK2::advance_timestep_impl).
 * Reference file:line citations are relative to the pbosler/lpm source tree.
 *
 * Conventions
 *  - All array pointers are DEVICE pointers owned by the caller; nothing is
 *    retained after a call returns (steppers keep only their own workspace).
 *  - Coordinates and vectors are passed as strided views (lpm_view): element
 *    (i, c) lives at p[i * stride_i + c * stride_c].  Kokkos LayoutRight (AoS)
 *    is stride_i = ndim, stride_c = 1; LayoutLeft (SoA, the Kokkos-CUDA default
 *    for View<Real*[3]>) is stride_i = 1, stride_c = nmax.
 *  - Masks are one byte per face slot, nonzero = divided face (excluded as a
 *    source), as View<bool*> in the reference.
 *  - Real = double, Index = 64-bit here (the reference uses int).
 *  - Calls are asynchronous and ordered on the context's CUDA stream, except
 *    where a host result is returned (invariants, error norms, timing).
 *  - Every call returns LPM_OK (0) or a negative code; lpm_last_error() gives
 *    a message (thread-local).  The C++ facade (lpm_gb300.hpp) turns nonzero
 *    codes into std::runtime_error, as LPM_REQUIRE does
 *    (src/lpm_assert.hpp:22-30).
 *  - One context per host thread; a context is not thread-safe.
 */
#ifndef LPM_GB300_H
#define LPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LPM_OK 0
#define LPM_ERR_ARG (-1)     /* invalid argument (null pointer, size, stride) */
#define LPM_ERR_CUDA (-2)    /* CUDA runtime error */
#define LPM_ERR_TIMEOUT (-3) /* a bounded device-side wait gave up */
#define LPM_ERR_ALLOC (-4)   /* device allocation failed */
#define LPM_ERR_STATE (-5)   /* object used in the wrong state */

/* ---- arithmetic of the pairwise sum ------------------------------------ */
/* LPM_FP64: the reference's pair kernels in FP64 (1 - x.y [+ eps^2] on the
 *            sphere, |x-y|^2 + eps^2 on the plane) with the cross product
 *            taken out of the sum (u = x cross sum_j (g_j / arg_j) y_j) and one
 *            Newton-Raphson quotient per pair; within 1e-12 of the reference.
 * LPM_FP64_EXACT: every pair term in FP64 in the reference's evaluation
 *            order (correctly rounded divisions), each term equal to the
 *            reference's bit for bit; about 3x slower than LPM_FP64.
 * LPM_FP32C: FP32 pair kernel (denominator rebuilt as |x-y|^2/2 + eps^2),
 *            per-tile Kahan/TwoSum-compensated sums, FP64 epilogue. */
#define LPM_FP64 64
#define LPM_FP64_EXACT 66
#define LPM_FP32C 32
/* LPM_FP64_CHORD: the LPM_FP32C algorithm (chord denominator, cross product
 * hoisted out of the sum) in FP64.  On unit vectors it equals LPM_FP64 to
 * rounding; off the sphere (RK stage positions, which leave the sphere by
 * O(dt^2 |u|^2)) it keeps evaluating the sphere kernel, where the reference's
 * 1 - x.y + eps^2 can turn non-positive. */
#define LPM_FP64_CHORD 65

/* geometry */
#define LPM_PLANE 2
#define LPM_SPHERE 3

typedef struct {
  double* p;
  int64_t stride_i;
  int64_t stride_c;
} lpm_view;

typedef struct lpm_context lpm_context;

/* ---- context ----------------------------------------------------------- */
/* Binds a CUDA device.  The context owns cached device scratch (packed source
 * tiles, per-chunk partial sums) that grows on demand. */
int lpm_context_create(lpm_context** ctx, int device);
int lpm_context_destroy(lpm_context* ctx);
/* cudaStream_t passed as void*; 0 = the legacy default stream. */
int lpm_context_set_stream(lpm_context* ctx, void* cuda_stream);
/* LPM_FP64 (default), LPM_FP64_EXACT, LPM_FP64_CHORD or LPM_FP32C for the
 * functor entry points below. */
int lpm_context_set_precision(lpm_context* ctx, int precision);
/* Fixes the FP32 N-body kernel shape (0-5: 256x4 with 3 or 4 CTAs per SM,
 * 128x8 with 4, 256x2 with 5, 128x8 with 3, 256x4 with 2; the same table as
 * lpm_ensemble_set_kernel) of later LPM_FP32C functor calls and of steppers
 * created afterwards (a stepper keeps the shape it was created with), or (-1,
 * the default) lets each problem size time the six shapes once and keep the
 * fastest.  A target's sums do not depend on the
 * shape. */
int lpm_context_set_kernel_shape(lpm_context* ctx, int shape);
/* Waits for the context's stream, then reports LPM_ERR_TIMEOUT if a bounded
 * device-side wait gave up since the last check (and clears the flag). */
int lpm_context_synchronize(lpm_context* ctx);
/* Number of CUDA kernels this context has launched so far. */
int64_t lpm_context_kernel_launches(const lpm_context* ctx);
/* Thread-local message for the last failing call on this thread. */
const char* lpm_last_error(void);
/* 1 if the library was built for the GPU in this process, 0 otherwise. */
int lpm_device_count(void);

/* ---- BVE direct sums on the sphere (src/lpm_bve_sphere_kernels.hpp) ----- */
/* BVEVertexSolve (:90-132): psi (nullable) and u (u.p nullable) at nverts
 * vertex targets from nfaces face slots (vorticity zeta, area, mask). */
int lpm_bve_vertex_solve(lpm_context* ctx, double* psi, lpm_view u,
                         lpm_view vx, int64_t nverts, lpm_view fx,
                         const double* zeta, const double* area,
                         const uint8_t* mask, int64_t nfaces);
/* BVEVertexStreamFn (:141-170). */
int lpm_bve_vertex_stream_fn(lpm_context* ctx, double* psi, lpm_view vx,
                             int64_t nverts, lpm_view fx, const double* zeta,
                             const double* area, const uint8_t* mask,
                             int64_t nfaces);
/* BVEVertexVelocity (:179-211). */
int lpm_bve_vertex_velocity(lpm_context* ctx, lpm_view u, lpm_view vx,
                            int64_t nverts, lpm_view fx, const double* zeta,
                            const double* area, const uint8_t* mask,
                            int64_t nfaces);
/* No counterpart in the reference.  BVEVertexVelocity in LPM_FP32C for
 * callers that cannot allocate device memory: it calls no cudaMalloc or
 * cudaFree and needs no context.  Its scratch is one 64 MiB array inside the
 * library, held on every GPU that loads it until the process exits; problems
 * needing more (about 40 B per face slot + 44 B per target) are rejected with
 * LPM_ERR_ARG.  The first call on a device looks up the array's address; make
 * it before any stream capture.  Calls share the array: calls that overlap on
 * the GPU race.  Runs on `cuda_stream` and returns after it has finished. */
int lpm_bve_vertex_velocity_static(lpm_view u, lpm_view vx, int64_t nverts,
                                   lpm_view fx, const double* zeta,
                                   const double* area, const uint8_t* mask,
                                   int64_t nfaces, void* cuda_stream);
/* BVEFaceSolve (:284-320): collocated face targets, i == j skipped. */
int lpm_bve_face_solve(lpm_context* ctx, double* psi, lpm_view u, lpm_view fx,
                       const double* zeta, const double* area,
                       const uint8_t* mask, int64_t nfaces);
/* BVEFaceStreamFn (:329-356). */
int lpm_bve_face_stream_fn(lpm_context* ctx, double* psi, lpm_view fx,
                           const double* zeta, const double* area,
                           const uint8_t* mask, int64_t nfaces);
/* BVEFaceVelocity (:365-394). */
int lpm_bve_face_velocity(lpm_context* ctx, lpm_view u, lpm_view fx,
                          const double* zeta, const double* area,
                          const uint8_t* mask, int64_t nfaces);
/* BVEVorticityTendency (:399-413): dzeta(i) = -2*Omega*u(i,2)*dt. */
int lpm_bve_vorticity_tendency(lpm_context* ctx, double* dzeta, lpm_view u,
                               int64_t n, double dt, double Omega);

/* ---- incompressible2d (src/lpm_incompressible2d_kernels.hpp) ----------- */
/* Incompressible2DPassiveSums<Geo> (:144-193); ndim = LPM_SPHERE or
 * LPM_PLANE; u.p and psi nullable. */
int lpm_ic2d_passive_sums(lpm_context* ctx, int ndim, lpm_view u, double* psi,
                          lpm_view x, int64_t n_passive, lpm_view y,
                          const double* zeta, const double* area,
                          const uint8_t* mask, double eps, int64_t n_active);
/* Incompressible2DActiveSums<Geo> (:201-246).  As in the reference the
 * i == j term is skipped only when eps is zero (:235); self_rule = 1 skips it
 * always (the rule of the BVE face functors). */
int lpm_ic2d_active_sums(lpm_context* ctx, int ndim, lpm_view u, double* psi,
                         lpm_view xy, const double* zeta, const double* area,
                         const uint8_t* mask, double eps, int64_t n_active,
                         int self_rule);
/* Incompressible2DTendencies<Geo> (:257-278): dzeta = -dfdt(u), with
 * CoriolisSphere(Omega) or CoriolisBetaPlane(f0, beta) (src/lpm_coriolis.hpp
 * :97-195); cor = Omega (sphere) or beta (plane). */
int lpm_ic2d_tendencies(lpm_context* ctx, int ndim, double* dzeta, lpm_view u,
                        int64_t n, double cor);
/* Incompressible2D::total_vorticity/total_enstrophy/total_kinetic_energy
 * (src/lpm_incompressible2d_impl.hpp:91-137), FP64, deterministic order.
 * out[0] = sum zeta*A, out[1] = 0.5 sum zeta^2 A, out[2] = 0.5 sum |u|^2 A
 * over unmasked faces.  Synchronous. */
int lpm_ic2d_invariants(lpm_context* ctx, int ndim, int64_t nfaces,
                        const double* zeta, lpm_view vel, const double* area,
                        const uint8_t* mask, double out[3]);

/* SphereTangentFunctor (src/lpm_sphere_functions.hpp:59-78): udotx(i) =
 * x(i,:) . u(i,:), the tangency diagnostic of a sphere velocity field. */
int lpm_sphere_tangency(lpm_context* ctx, double* udotx, lpm_view x, lpm_view u,
                        int64_t n);

/* ---- ErrNorms (src/lpm_error.hpp:81-91) -------------------------------- */
/* Relative l1, l2 (weighted by wt; wt may be null = 1) and linf
 * (max|err|/max|exact|) of vector magnitudes (ndim > 1) or values (ndim 1);
 * mask (nullable) excludes entries.  Synchronous. */
int lpm_err_norms(lpm_context* ctx, int ndim, int64_t n, lpm_view appx,
                  lpm_view exact, const double* wt, const uint8_t* mask,
                  double out[3]);

/* ---- steppers ---------------------------------------------------------- */
/* Step options (bit flags). */
#define LPM_STEP_FIX_FACEVORT3 1u /* BVE: use stage-3 face vorticity in the
                                     final update; the reference passes
                                     facevort4 twice
                                     (src/lpm_bve_rk4_impl.hpp:155-157) */
#define LPM_STEP_REPROJECT 2u     /* renormalise positions to the unit sphere
                                     after each step (the reference does not) */
#define LPM_STEP_SKIP_MASKED_TARGETS 4u /* do not evaluate, nor move, divided
                                     (masked) face slots; the reference
                                     evaluates them although nothing reads
                                     their values */
#define LPM_STEP_SKIP_SELF_ALWAYS 8u /* ic2d: skip i == j also for eps > 0 */
#define LPM_STEP_NO_GRAPH 16u     /* launch stages directly instead of
                                     replaying a captured CUDA graph */
#define LPM_STEP_TIME_NBODY 32u   /* bracket every N-body launch with CUDA
                                     events (implies LPM_STEP_NO_GRAPH); read
                                     with lpm_*_nbody_time */

typedef struct lpm_bve_rk4 lpm_bve_rk4;
/* BVERK4(dt, sphere) + BVERK4::init (src/lpm_bve_rk4.hpp:10-77,
 * src/lpm_bve_rk4.cpp:5-39): allocates the stage workspace for nverts
 * vertices and nfaces face slots.  precision: LPM_FP64 or LPM_FP32C. eps is
 * the kernel smoothing (0 = the reference BVE functors). */
int lpm_bve_rk4_create(lpm_context* ctx, lpm_bve_rk4** out, int64_t nverts,
                       int64_t nfaces, double dt, double Omega, double eps,
                       int precision, uint32_t flags);
int lpm_bve_rk4_destroy(lpm_bve_rk4* st);
/* BVERK4::advance_timestep (src/lpm_bve_rk4_impl.hpp:55-167): advances
 * positions and relative vorticity of vertices and faces by one RK4 step and
 * leaves the velocities of the new state in vvel/fvel (which must hold the
 * velocities of the current state on entry, as after
 * BVESphere::init_velocity).  farea/fmask must not change between calls. */
int lpm_bve_rk4_advance_timestep(lpm_bve_rk4* st, lpm_view vx, double* vzeta,
                                 lpm_view vvel, lpm_view fx, double* fzeta,
                                 lpm_view fvel, const double* farea,
                                 const uint8_t* fmask);

/* With LPM_STEP_TIME_NBODY: total device time (ms) and number of the N-body
 * launches since the previous call (then reset).  Synchronous. */
int lpm_bve_rk4_nbody_time(lpm_bve_rk4* st, double* ms, int64_t* launches);
/* The N-body kernel shape the stepper runs: threads per CTA, targets per
 * thread and the CTAs per SM its register cap is set for (LPM_FP32C: the
 * autotuned one of the six shapes; FP64 forms: the fixed shape, 0 CTAs).
 * Valid after the first step (LPM_ERR_STATE before). */
int lpm_bve_rk4_kernel_shape(lpm_bve_rk4* st, int* threads, int* targets_per_thread,
                             int* min_ctas_per_sm);

typedef struct lpm_ic2d_rk2 lpm_ic2d_rk2;
/* Incompressible2DRK2(dt, ic2d) (src/lpm_incompressible2d_rk2_impl.hpp:15-43).
 * ndim = LPM_SPHERE or LPM_PLANE; cor = Coriolis Omega or beta. */
int lpm_ic2d_rk2_create(lpm_context* ctx, lpm_ic2d_rk2** out, int ndim,
                        int64_t nverts, int64_t nfaces, double dt, double eps,
                        double cor, int precision, uint32_t flags);
int lpm_ic2d_rk2_destroy(lpm_ic2d_rk2* st);
/* Incompressible2DRK2::advance_timestep_impl (:74-172).  vvel/fvel/vpsi/fpsi
 * hold the sums of the current state on entry (as after
 * Incompressible2D::init_direct_sums) and of the new state on exit. */
int lpm_ic2d_rk2_advance_timestep(lpm_ic2d_rk2* st, lpm_view vx,
                                  double* vzeta, lpm_view vvel, double* vpsi,
                                  lpm_view fx, double* fzeta, lpm_view fvel,
                                  double* fpsi, const double* farea,
                                  const uint8_t* fmask);
int lpm_ic2d_rk2_nbody_time(lpm_ic2d_rk2* st, double* ms, int64_t* launches);

/* ---- one-call forms ------------------------------------------------------ */
/* For hosts that keep no lpm_context: coordinate views with their count, a
 * precision (LPM_FP64, LPM_FP64_CHORD or LPM_FP32C) and a CUDA stream (NULL =
 * the legacy default stream).  A context cached per host thread and device
 * does the work, stream-ordered; switching streams synchronises the previous
 * one (the cached context's scratch memory is reused by the next call).
 * want: 1 = velocity, 2 = stream function, 3 = both.  collocated: the
 * targets are the sources (the same view, n == n_src).
 * lpm_bve_direct_sum: eps == 0 gives the BVE functors (BVEVertexSolve /
 * BVEFaceSolve arithmetic, collocated targets skip i == j); eps > 0 the
 * smoothed sphere kernel of Incompressible2DKernels with the same i == j
 * rule.  lpm_plane_direct_sum: the planar Incompressible2D sums (collocated
 * targets skip i == j only when eps is zero, as Incompressible2DActiveSums). */
typedef struct {
  const double* p;
  long long n;
  long long stride_i;
  long long stride_c;
} lpm_crd3;
int lpm_bve_direct_sum(lpm_crd3 tgt, lpm_crd3 src, const double* zeta,
                       const double* area, const unsigned char* mask,
                       long long n_src, int collocated, double eps, int want,
                       int precision, double* u_out, long long u_stride_i,
                       long long u_stride_c, double* psi_out,
                       void* cuda_stream);
int lpm_plane_direct_sum(lpm_crd3 tgt, lpm_crd3 src, const double* zeta,
                         const double* area, const unsigned char* mask,
                         long long n_src, int collocated, double eps, int want,
                         int precision, double* u_out, long long u_stride_i,
                         long long u_stride_c, double* psi_out,
                         void* cuda_stream);
/* Frees the calling thread's cached contexts (all devices) after
 * synchronising their streams; the next one-call form creates a new one.
 * Call it before a host thread that used the one-call forms exits. */
int lpm_one_call_release(void);
/* One step of a stepper (the advance_timestep calls above under the step
 * names), and nsteps RK4 steps of every problem of an ensemble. */
int lpm_bve_rk4_step(lpm_bve_rk4* st, lpm_view vx, double* vzeta,
                     lpm_view vvel, lpm_view fx, double* fzeta, lpm_view fvel,
                     const double* farea, const uint8_t* fmask);
int lpm_ic2d_rk2_step(lpm_ic2d_rk2* st, lpm_view vx, double* vzeta,
                      lpm_view vvel, double* vpsi, lpm_view fx, double* fzeta,
                      lpm_view fvel, double* fpsi, const double* farea,
                      const uint8_t* fmask);

/* ---- ensembles of independent BVE problems ----------------------------- */
/* No single reference counterpart: many BVESphere/BVERK4 instances advanced
 * together.  Problem p owns nverts[p] vertex rows and nfaces[p] face-slot
 * rows of the concatenated arrays (problem 0 first).  fmask: device, all
 * face slots (fixed).  precision: LPM_FP32C or LPM_FP64_CHORD (chord form,
 * velocity only).  Each evaluation is one persistent launch over (problem,
 * target block, source chunk) work items; a step is replayed from a CUDA
 * graph; the chunk length, the FP32 kernel shape (threads x targets per
 * thread) and the launch form (persistent or one CTA per item) are autotuned
 * on the first call. */
typedef struct lpm_ensemble lpm_ensemble;
int lpm_ensemble_create(lpm_context* ctx, lpm_ensemble** out, int nproblems,
                        const int64_t* nverts, const int64_t* nfaces,
                        const uint8_t* fmask, double dt, double Omega,
                        double eps, int precision, uint32_t flags);
int lpm_ensemble_destroy(lpm_ensemble* e);
/* Velocities of the current state of every problem (one evaluation). */
int lpm_ensemble_velocity(lpm_ensemble* e, lpm_view vx, lpm_view vvel,
                          lpm_view fx, const double* fzeta, lpm_view fvel,
                          const double* farea);
/* One RK4 step of every problem (BVERK4::advance_timestep semantics). */
int lpm_ensemble_advance_timestep(lpm_ensemble* e, lpm_view vx, double* vzeta,
                                  lpm_view vvel, lpm_view fx, double* fzeta,
                                  lpm_view fvel, const double* farea);
/* Autotuned chunk length (sources), work items per evaluation, padded
 * targets. */
int lpm_ensemble_info(lpm_ensemble* e, int64_t* chunk_len, int64_t* items,
                      int64_t* targets);
int lpm_ensemble_nbody_time(lpm_ensemble* e, double* ms, int64_t* launches);
/* Kernel in use: threads per CTA, targets per thread and the launch form
 * (persistent: 1 = persistent CTAs drain the work list, 0 = one CTA per work
 * item, longest first; nullable). */
int lpm_ensemble_shape(lpm_ensemble* e, int* threads, int* targets_per_thread,
                       int* persistent);
/* Fixes the FP32 kernel shape (0-5, as for lpm_context_set_kernel_shape)
 * and the launch form (persistent 1 or one CTA per item 0); with
 * lpm_ensemble_set_chunk_len, instead of autotuning.  Results do not depend
 * on either.  Call before the first velocity/step call. */
int lpm_ensemble_set_kernel(lpm_ensemble* e, int shape, int persistent);
/* Fixes the chunk length (sources; rounded up to whole tiles) instead of
 * autotuning it, e.g. for bitwise-reproducible runs across ensembles.  Call
 * before the first velocity/step call. */
int lpm_ensemble_set_chunk_len(lpm_ensemble* e, int64_t chunk_len);
int lpm_ensemble_run(lpm_ensemble* e, int nsteps, lpm_view vx, double* vzeta,
                     lpm_view vvel, lpm_view fx, double* fzeta, lpm_view fvel,
                     const double* farea);

/* ---- host-side inputs: meshes and initial conditions -------------------- */
/* Mesh kinds (restatements of the reference seeds' tree_init,
 * src/mesh/lpm_polymesh2d_impl.hpp:26-42, with the triangle and quad dividers
 * of src/mesh/lpm_faces_impl.hpp:285-575). */
#define LPM_MESH_ICOS_TRI 1     /* IcosTriSphereSeed */
#define LPM_MESH_CUBED_SPHERE 2 /* CubedSphereSeed */
#define LPM_MESH_QUAD_RECT 3    /* QuadRectSeed, [-radius, radius]^2 */
/* Vertex count and face-slot count (all tree levels) for a uniform mesh. */
int lpm_mesh_sizes(int kind, int level, int64_t* nverts, int64_t* nfaces);
/* Fills HOST arrays: vx (nverts x ndim, AoS), fx (nfaces x ndim, AoS),
 * farea (nfaces), fmask (nfaces; 1 = divided parent slot, area 0).  Face
 * slots are ordered like the reference's tree (seed faces, then four children
 * per divided face, level by level). */
int lpm_mesh_build(int kind, int level, double radius, double* vx, double* fx,
                   double* farea, uint8_t* fmask);

/* The same mesh built on the device (uniform refinement in parallel, one
 * level per pass): DEVICE arrays of lpm_mesh_sizes' sizes.  Positions equal
 * lpm_mesh_build's bit for bit; areas to the last bits of tan/atan. */
int lpm_mesh_build_device(lpm_context* ctx, int kind, int level, double radius,
                          double* vx, double* fx, double* farea, uint8_t* fmask);

/* Initial vorticity kinds (src/lpm_vorticity_gallery.hpp). */
#define LPM_IC_SOLID_BODY 1      /* SolidBodyRotation: 2*OMEGA*z, OMEGA=2pi */
#define LPM_IC_GAUSSIAN_SPHERE 2 /* params: strength, b, lon, lat, gauss_const,
                                    background_Omega (adds 2*Omega*z) */
#define LPM_IC_RH54 3            /* RossbyHaurwitz54: params u0, amplitude */
#define LPM_IC_DIPOLE_PAIR 4     /* CollidingDipolePairPlane: strA, rA, xA, yA,
                                    strB, rB, xB, yB */
#define LPM_IC_MULTI_GAUSSIAN 5  /* sum of k Gaussians: params k, then per
                                    vortex (strength, b, lon, lat) */
/* Evaluates relative vorticity at n HOST points x (n x ndim, AoS). */
int lpm_ic_eval(int kind, const double* params, int nparams, int ndim,
                int64_t n, const double* x, double* zeta);

/* ---- instrumentation ----------------------------------------------------- */
/* Test of the failure path, no counterpart in the reference (whose device
 * checks abort, src/lpm_assert.hpp:32-46).  Launches one CTA on the context's
 * stream whose tile wait cannot complete (its mbarrier expects a copy that is
 * never issued); after spin_limit polls (1 to 2^20) it sets the context's
 * timeout flag and returns without touching global memory, exactly as an
 * N-body kernel does when a tile copy never lands.  The next
 * lpm_context_synchronize reports LPM_ERR_TIMEOUT and clears the flag; the
 * context stays usable. */
int lpm_wait_selftest(lpm_context* ctx, int spin_limit);
/* Measured FP32 / FP64 FMA peak of this GPU (TFLOP/s) from a short
 * register-only microbenchmark; synchronous. */
int lpm_measure_fma_peak(lpm_context* ctx, int precision, double* tflops);

/* ---- planar shallow-water direct sums ------------------------------------ */
/* PlanarSWEVertexSums (src/lpm_swe_kernels.hpp:626-721): at nv vertices vx
 * (nv x 2) with surface height vs, from the face slots fx/fzeta/fsigma/
 * farea/fmask/fs (nf): velocity u (written if do_velocity), the double dot
 * product du/dx^2 + 2 du/dy dv/dx + dv/dy^2, the four velocity gradients,
 * the PSE surface Laplacian (pse::BivariateOrder8 of width pse_eps), the
 * stream and potential functions; masked faces are skipped.  Context
 * precision LPM_FP64: the reference's pair arithmetic (planar_swe_sums_rhs_pse,
 * :394-480); LPM_FP32C: FP32 moment sums with compensation (velocity ~1e-7,
 * stream/potential ~1e-6, gradients and Laplacian ~1e-5 relative). */
int lpm_swe_plane_vertex_sums(lpm_context* ctx, lpm_view u, double* ddot,
                              double* du1dx1, double* du1dx2, double* du2dx1,
                              double* du2dx2, double* laps, double* psi,
                              double* phi, lpm_view vx, const double* vs,
                              int64_t nv, lpm_view fx, const double* fzeta,
                              const double* fsigma, const double* farea,
                              const uint8_t* fmask, const double* fs, int64_t nf,
                              double eps, double pse_eps, int do_velocity);
/* PlanarSWEFaceSums (:787-876): the same at every face slot; for
 * |eps| < DBL_EPSILON the i == j pair is skipped (collocated =
 * FloatingPoint<Real>::zero(eps)). */
int lpm_swe_plane_face_sums(lpm_context* ctx, lpm_view u, double* ddot,
                            double* du1dx1, double* du1dx2, double* du2dx1,
                            double* du2dx2, double* laps, double* psi,
                            double* phi, lpm_view fx, const double* fzeta,
                            const double* fsigma, const double* farea,
                            const uint8_t* fmask, const double* fs, int64_t nf,
                            double eps, double pse_eps, int do_velocity);

/* ---- spherical shallow-water direct sums --------------------------------- */
/* SphereVertexSums (src/lpm_swe_kernels.hpp:723-785): at nv vertices vx
 * (nv x 3), from the face slots fx/fzeta/fsigma/farea/fmask (nf): velocity u
 * (nv x 3, written if do_velocity) of kzeta_sphere + ksigma_sphere and the
 * double dot product sum_ij M_ij M_ji of the summed gradient tensor
 * M = sum_j grad_kzeta rot_j + grad_ksigma pot_j (rot = -zeta A,
 * pot = -sigma A; sphere_swe_velocity_sums, :335-373).  grad, if not NULL,
 * receives M itself (nv x 9, row-major, contiguous).  Masked faces are
 * skipped.  Context precision LPM_FP64 (or LPM_FP64_CHORD): FP64, the
 * reference's pair arithmetic; LPM_FP32C: FP32 chord-form moments with
 * compensated sums (velocity ~1e-7, gradient ~1e-5 relative). */
int lpm_swe_sphere_vertex_sums(lpm_context* ctx, lpm_view u, double* ddot,
                               double* grad, lpm_view vx, int64_t nv,
                               lpm_view fx, const double* fzeta,
                               const double* fsigma, const double* farea,
                               const uint8_t* fmask, int64_t nf, double eps,
                               int do_velocity);
/* SphereFaceSums (:877-940): the same at every face slot; for
 * |eps| < DBL_EPSILON the i == j pair is skipped. */
int lpm_swe_sphere_face_sums(lpm_context* ctx, lpm_view u, double* ddot,
                             double* grad, lpm_view fx, const double* fzeta,
                             const double* fsigma, const double* farea,
                             const uint8_t* fmask, int64_t nf, double eps,
                             int do_velocity);

/* ---- mesh connectivity and VTK output (host) ----------------------------- */
/* Face vertex lists of the uniform mesh lpm_mesh_build makes: *nfv vertices
 * per face slot (3 icosahedral, 4 cubed sphere / quad), counter-clockwise
 * seen from outside (sphere) or from +z (plane), parents included.  With
 * fverts == NULL only *nfv is set; otherwise fverts holds nfaces * nfv. */
int lpm_mesh_face_vertices(int kind, int level, double radius, int* nfv,
                           int32_t* fverts);

/* One data array of a VTK file: location 0 = point data (one tuple per
 * vertex), 1 = cell data (one tuple per face slot; leaf slots written);
 * ncomp values per tuple, row-major. */
typedef struct {
  const char* name;
  int location;
  int ncomp;
  const double* data;
} lpm_vtk_field;

/* VtkPolymeshInterface (src/vtk/lpm_vtk_io.hpp:36-76) without VTK: writes a
 * VTK XML PolyData file (.vtp, ASCII, shortest round-trip decimals) of the
 * vertices (points; z = height in the plane, (1 + height) x on the sphere
 * when height is not NULL) and the leaf faces (polygons, slot order), cell
 * array "area", then the fields in order.  All pointers are host memory. */
int lpm_vtk_write_polymesh(const char* path, int ndim, int64_t nv,
                           const double* vx, const double* height, int64_t nf,
                           int nfv, const int32_t* fverts, const uint8_t* fmask,
                           const double* farea, int nfields,
                           const lpm_vtk_field* fields);

/* NcWriter (src/netcdf/lpm_netcdf_writer.cpp:5-47) with the mesh and field
 * content of the reference's NetCDF definitions (src/netcdf/lpm_netcdf_impl.hpp),
 * without the netCDF library: writes a classic-format NetCDF file (64-bit
 * offsets, CDF-2) with the global attribute LPM, an unlimited "time"
 * dimension holding one record (time, vertices.phys_crds, faces.phys_crds and
 * the fields, named by the caller: location 0 = vertices, 1 = face slots;
 * 1 or ndim components), and the fixed arrays faces.vertices (int),
 * faces.mask (byte) and faces.area.  All pointers are host memory. */
int lpm_netcdf_write_polymesh(const char* path, int ndim, int64_t nv,
                              const double* vx, int64_t nf, int nfv,
                              const int32_t* fverts, const uint8_t* fmask,
                              const double* farea, const double* fx, double time,
                              int nfields, const lpm_vtk_field* fields);

/* ---- octree far field with a learned correction ------------------------- */
/* No reference counterpart: the reference's octree sources (LpmOctree*,
 * LpmNodeArray*) are not built and src/tree/lpm_cpu_tree's generators are
 * never called.  This is an alternative evaluator of the BVE sphere velocity
 * (the sum of BVEVertexVelocity / BVEFaceVelocity, chord form with smoothing
 * eps): an octree over the sources (leaves of <= leaf_max points), a target
 * block of 128 Morton-ordered targets accepts a cell when
 * h <= theta * (distance - block radius); accepted cells use the order-4
 * Cartesian expansion of the kernel about the cell centre, the rest of the
 * tree down to the leaves is summed exactly (FP32 compensated).  With a
 * trained network enabled, every accepted cell with h / (distance - block
 * radius) >= rho_min also gets the network's prediction of the expansion's
 * residual (BF16 MLP on tcgen05 tensor cores).  A target block whose
 * interaction lists overflow falls back to the full direct sum. */
#define LPM_FF_NPARAM 40960 /* FP32 master weights: W1 128x48, W2 128x128,
                               W3 128x128, W4 16x128, row-major */
#define LPM_FF_NNORM 97     /* input mean[48], input 1/std[48], output scale */
#define LPM_FF_NIN 48       /* network inputs (feature 40 is the constant 1) */
typedef struct lpm_farfield lpm_farfield;
int lpm_farfield_create(lpm_context* ctx, lpm_farfield** out, double theta,
                        int leaf_max, double rho_min);
int lpm_farfield_destroy(lpm_farfield* ff);
/* Velocity at nx targets x (device, strided) from the face slots fx/zeta/
 * area/mask (nf slots, the BVEFaceVelocity source arguments).  Builds the
 * tree for these positions (host sort, synchronises) and evaluates. */
int lpm_farfield_velocity(lpm_farfield* ff, lpm_view u, lpm_view x,
                          int64_t nx, lpm_view fx, const double* zeta,
                          const double* area, const uint8_t* mask, int64_t nf,
                          double eps);
/* Trains the network on nsamples (cell, target) samples drawn from seeded
 * random vortex fields on icosahedral meshes of levels level_min..level_max
 * (the exact FP64 cell sum minus the expansion is the target), with Adam,
 * cosine learning rate, the given batch (a multiple of 128) and epochs.
 * loss (optional, epochs floats) receives the mean loss per epoch.  Enables
 * the network. */
int lpm_farfield_train(lpm_farfield* ff, int64_t nsamples, int epochs,
                       int batch, double lr, uint64_t seed, int level_min,
                       int level_max, double eps, float* loss);
int lpm_farfield_set_network(lpm_farfield* ff, int enable);
/* HOST buffers of LPM_FF_NPARAM and LPM_FF_NNORM floats. */
int lpm_farfield_get_weights(lpm_farfield* ff, float* w, float* norm);
int lpm_farfield_set_weights(lpm_farfield* ff, const float* w,
                             const float* norm);
/* Gradient of the mean squared error (sum over the 3 outputs, mean over n
 * rows, n a multiple of 128) with respect to the master weights, from the
 * tensor-core training kernel: x = HOST n x 48 normalised inputs (rounded to
 * BF16), y = HOST n x 3 targets, grad = HOST LPM_FF_NPARAM floats. */
int lpm_farfield_grad(lpm_farfield* ff, const float* x, const float* y, int n,
                      float* grad);
/* Of the last evaluation: far (block, cell) pairs, near (target, source)
 * pairs / 128, learned (block, cell) pairs, blocks on the direct-sum
 * fallback, cells, target blocks, (target, cell) rows the network evaluated.
 * out: 7 int64.  Synchronous. */
int lpm_farfield_stats(lpm_farfield* ff, int64_t* out);
/* Device time of the evaluations since the previous call (tree kernels and
 * network kernel, ms) and their count, then resets; enable != 0 brackets the
 * following evaluations with CUDA events (use with LPM_STEP_TIME_NBODY
 * steppers or direct calls, not inside graph capture).  Synchronous. */
int lpm_farfield_timing(lpm_farfield* ff, int enable, double* tree_ms,
                        double* net_ms, int64_t* evals);
/* Evaluate BVERK4 stages with the far field instead of the direct sum
 * (precision LPM_FP64_CHORD steppers; the tree is built on the first step and
 * rebuilt every rebuild_every steps, 0 = never).  ff must outlive st. */
int lpm_bve_rk4_set_farfield(lpm_bve_rk4* st, lpm_farfield* ff,
                             int rebuild_every);
/* Host only (no GPU): builds the octree of nsrc sources and the target blocks
 * of ntgt targets (HOST n x 3 arrays) and summarises them in out[9]: cells,
 * leaves, largest leaf, deepest level, target blocks, smallest block fill,
 * targets covered, sources in leaves, and the count of structural errors
 * (permutation, child ranges, duplicate targets) -- 0 for a valid tree. */
int lpm_octree_stats(const double* src_xyz, int64_t nsrc, const double* tgt_xyz,
                     int64_t ntgt, int leaf_max, int64_t* out);
/* tcgen05 operand-layout self-test: D (128 x N) = A * B on the tensor cores,
 * A 128 x K (a_mn = 0) or K x 128 (a_mn = 1), B N x K (b_mn = 0) or K x N
 * (b_mn = 1), row-major FP32 device arrays rounded to BF16; N, K multiples of
 * 16 in [16, 128]. */
int lpm_tc_selftest(lpm_context* ctx, const float* A, const float* B, float* D,
                    int N, int K, int a_mn, int b_mn);

#ifdef __cplusplus
}
#endif

#endif /* LPM_GB300_H */

// stepper.cu -- device-resident time steppers.
//
// BVERK4::advance_timestep (src/lpm_bve_rk4_impl.hpp:63-167) runs, per step,
// 4 direct-sum evaluations plus ~30 BLAS-1 / tendency launches.  Here every
// O(N) operation between two evaluations is fused into the epilogue that
// combines the previous evaluation's partial sums: it writes the velocity,
// forms the stage increments (KokkosBlas::scal, BVEVorticityTendency), the
// next stage's work positions and vorticity (KokkosBlas::update), and packs
// the next evaluation's source and target tiles.  A step is then
//   begin, [nbody, stage] x 3, nbody, final
// = 9 kernels, captured once into a CUDA graph and replayed.
//
// All state updates are FP64 with non-contracting intrinsics in the
// reference's operation order; only the pair sums use the FP32 form when the
// stepper runs in LPM_FP32C.
//
// Incompressible2DRK2::advance_timestep_impl
// (src/lpm_incompressible2d_rk2_impl.hpp:74-172) is fused the same way:
//   begin, nbody, mid, nbody, final.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lpm_host.hpp"
#include "nbody.cuh"
#include "farfield.hpp"
#include "stage.cuh"


// ---------------------------------------------------------------------------
// Common stepper state
// ---------------------------------------------------------------------------
struct lpm_stepper_base {
  lpm_context* ctx = nullptr;
  int ndim = 3;
  int64_t nv = 0, nf = 0;
  double dt = 0, eps = 0;
  int precision = LPM_FP64;
  uint32_t flags = 0;
  int form = lpm::FORM_BVE;
  bool skip_self = true;
  bool want_psi = false;

  bool ready = false;
  int64_t nsrc = 0, nft = 0, T = 0;
  lpm::NbodyPlan plan{};
  int shape_u = 0;  // FP32 shape of the velocity-only evaluation (RK2 stage)
  std::vector<void*> allocs;
  int *slot2src = nullptr, *src2slot = nullptr, *fslot = nullptr, *tself = nullptr;
  void *tgt = nullptr, *src = nullptr;
  double* part = nullptr;
  double* sgbuf = nullptr;  // [0] = sum, [8..] partials

  // optional octree far field in place of the direct sum (BVE, FP64 chord packs)
  lpm_farfield* ff = nullptr;
  int ff_every = 0;
  int64_t ff_steps = 0;

  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<char> key;
  int64_t graph_kernels = 0;

  void* dalloc(size_t bytes) {
    void* p = nullptr;
    LPM_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
    allocs.push_back(p);
    return p;
  }
  void free_all() {
    for (cudaEvent_t e : timers) cudaEventDestroy(e);
    timers.clear();
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    if (cap_stream) cudaStreamDestroy(cap_stream);
    cap_stream = nullptr;
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
  }

  // Maps, packed buffers and the launch plan; run once (the mask is fixed).
  void setup(const uint8_t* fmask) {
    lpm_context& c = *ctx;
    slot2src = static_cast<int*>(dalloc(sizeof(int) * nf));
    src2slot = static_cast<int*>(dalloc(sizeof(int) * nf));
    c.arena.reset();
    c.arena.reserve(sizeof(int) * (2 * size_t(nf) / 1024 + 8) + 4096);
    nsrc = lpm::compact_sources(c, fmask, nf, slot2src, src2slot);
    const bool skip_masked = flags & LPM_STEP_SKIP_MASKED_TARGETS;
    nft = skip_masked ? nsrc : nf;
    T = nv + nft;
    fslot = static_cast<int*>(dalloc(sizeof(int) * std::max<int64_t>(nft, 1)));
    if (nf > 0) {
      lpm::k_face_targets<<<(nf + 255) / 256, 256, 0, c.stream>>>(fmask, nf, skip_masked,
                                                                  slot2src, fslot);
      c.launches++;
    }
    plan = lpm::plan_nbody(c, precision, ndim, form, true, want_psi, T, nsrc);
    plan.skipc = skip_self;
    const size_t rec = precision == LPM_FP32C ? 16 : 32;  // float4 / double4_16a
    tgt = dalloc(rec * plan.ntgt_pad);
    src = dalloc(32 * plan.nsrc_pad);  // SrcF32 / double4_16a
    tself = static_cast<int*>(dalloc(sizeof(int) * plan.ntgt_pad));
    part = static_cast<double*>(dalloc(plan.part_bytes()));
    sgbuf = static_cast<double*>(dalloc(sizeof(double) * (8 + 256)));
    // zero the padding records once (never rewritten); tself padding = -1
    zero(tgt, rec * plan.ntgt_pad);
    zero(src, 32 * plan.nsrc_pad);
    LPM_CUDA(cudaMemsetAsync(tself, 0xff, sizeof(int) * plan.ntgt_pad, c.stream));
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    // kernel shape for this problem size (the zeroed tiles time like real ones)
    plan.shape = lpm::tune_shape(c, plan, tgt, tself, src, part, eps);
    shape_u = plan.shape;
    if (plan.wp) {  // the RK2 stage evaluation runs the velocity-only kernel
      lpm::NbodyPlan pu = plan;
      pu.wp = false;
      pu.ncomp = plan.ncomp - 1;
      shape_u = lpm::tune_shape(c, pu, tgt, tself, src, part, eps);
    }
    LPM_CUDA(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    ready = true;
  }
  void zero(void* p, size_t n) {
    lpm::k_zero_bytes<<<(n + 255) / 256, 256, 0, ctx->stream>>>(static_cast<char*>(p), n);
    ctx->launches++;
  }

  lpm::Tg targets(lpm_view vx, double* vzeta, lpm_view vvel, double* vpsi,
                  lpm_view fx, double* fzeta, lpm_view fvel, double* fpsi,
                  const double* farea) const {
    lpm::Tg g;
    g.ndim = ndim;
    g.nv = nv;
    g.T = T;
    g.fslot = fslot;
    g.slot2src = slot2src;
    g.vx = lpm::to_view(vx);
    g.fx = lpm::to_view(fx);
    g.vvel = lpm::to_view(vvel);
    g.fvel = lpm::to_view(fvel);
    g.vzeta = vzeta;
    g.fzeta = fzeta;
    g.vpsi = vpsi;
    g.fpsi = fpsi;
    g.farea = farea;
    return g;
  }
  double c0() const {
    return precision == LPM_FP32C ? double(lpm::f32_c0(ndim, eps)) : lpm::chord_c0(ndim, eps);
  }
  lpm::Pk packs() const {
    lpm::Pk k;
    k.mode = lpm::mode_of(precision);
    k.exact = lpm::ref64_exact(precision);
    k.form = form;
    k.skip_self = skip_self;
    k.tgt = tgt;
    k.tself = tself;
    k.src = src;
    k.part = part;
    k.nchunks = ff ? 1 : plan.nchunks;
    k.tpad = plan.ntgt_pad;
    return k;
  }
  // Builds the far field's tree from the current positions when it is due
  // (first step, then every ff_every steps); outside any graph capture.
  void ff_prepare(const lpm::Tg& g) {
    if (!ff) return;
    const bool due = !ff->built() || (ff_every > 0 && ff_steps % ff_every == 0);
    ff_steps++;
    if (!due) return;
    lpm_context& c = *ctx;
    c.arena.reset();
    c.arena.reserve(sizeof(double) * 3 * size_t(T + nsrc) + 4096);
    double* d = static_cast<double*>(c.arena.take(sizeof(double) * 3 * size_t(T + nsrc)));
    const int64_t n = T + nsrc;
    lpm::k_snapshot<<<unsigned((n + 255) / 256), 256, 0, c.stream>>>(g, src2slot, nsrc, d, d + 3 * T);
    c.launches++;
    std::vector<double> h(3 * size_t(n));
    LPM_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c.stream));
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    ff->build(h.data() + 3 * T, nsrc, h.data(), T);
  }
  // One N-body evaluation; with_psi = false evaluates the velocity only (a
  // plan without the stream-function component) even if the stepper wants psi.
  void nbody(bool with_psi = true) {
    const bool wp = want_psi && with_psi;
    lpm::NbodyPlan pl = plan;
    if (plan.wp && !wp) {
      pl.wp = false;
      pl.ncomp = plan.ncomp - 1;
      pl.shape = shape_u;
    }
    if (ff) {
      cudaEvent_t e[2];
      const bool timed = flags & LPM_STEP_TIME_NBODY;
      if (timed) {
        LPM_CUDA(cudaEventCreate(&e[0]));
        LPM_CUDA(cudaEventCreate(&e[1]));
        LPM_CUDA(cudaEventRecord(e[0], ctx->stream));
      }
      ff->evaluate(tgt, src, part, plan.ntgt_pad, c0(), eps);
      if (timed) {
        LPM_CUDA(cudaEventRecord(e[1], ctx->stream));
        timers.push_back(e[0]);
        timers.push_back(e[1]);
      }
      return;
    }
    if (lpm::mode_of(precision) != lpm::M_REF64 && wp && ndim == 3)
      lpm::sum_strengths(*ctx, src, precision == LPM_FP32C, nsrc, sgbuf, sgbuf + 8);
    if (flags & LPM_STEP_TIME_NBODY) {
      cudaEvent_t e[2];
      LPM_CUDA(cudaEventCreate(&e[0]));
      LPM_CUDA(cudaEventCreate(&e[1]));
      LPM_CUDA(cudaEventRecord(e[0], ctx->stream));
      lpm::launch_nbody(*ctx, pl, tgt, tself, src, part, eps);
      LPM_CUDA(cudaEventRecord(e[1], ctx->stream));
      timers.push_back(e[0]);
      timers.push_back(e[1]);
      return;
    }
    lpm::launch_nbody(*ctx, pl, tgt, tself, src, part, eps);
  }

  std::vector<cudaEvent_t> timers;
  // Sums and clears the recorded N-body timings.
  void nbody_time(double* ms, int64_t* n) {
    LPM_CUDA(cudaStreamSynchronize(ctx->stream));
    double tot = 0;
    for (size_t i = 0; i + 1 < timers.size(); i += 2) {
      float m = 0;
      LPM_CUDA(cudaEventElapsedTime(&m, timers[i], timers[i + 1]));
      tot += m;
    }
    *ms = tot;
    *n = int64_t(timers.size() / 2);
    for (cudaEvent_t e : timers) cudaEventDestroy(e);
    timers.clear();
  }

  // Runs `body` either directly or through a graph captured for this key.
  template <typename F>
  void run(const std::vector<char>& k, F body) {
    lpm_context& c = *ctx;
    if (flags & (LPM_STEP_NO_GRAPH | LPM_STEP_TIME_NBODY)) {
      body();
      LPM_CUDA(cudaGetLastError());
      return;
    }
    if (!exec || k != key) {
      if (exec) cudaGraphExecDestroy(exec);
      exec = nullptr;
      cudaStream_t user = c.stream;
      const int64_t before = c.launches;
      // order the capture after prior work on the user's stream
      LPM_CUDA(cudaStreamSynchronize(user));
      c.stream = cap_stream;
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        try {
          body();
        } catch (...) {
          cudaStreamEndCapture(cap_stream, &graph);
          if (graph) cudaGraphDestroy(graph);
          c.stream = user;
          throw;
        }
        e = cudaStreamEndCapture(cap_stream, &graph);
      }
      c.stream = user;
      LPM_CUDA(e);
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      LPM_CUDA(e);
      graph_kernels = c.launches - before;
      c.launches = before;
      key = k;
    }
    LPM_CUDA(cudaGraphLaunch(exec, c.stream));
    c.launches += graph_kernels;
  }
};

struct lpm_bve_rk4 : lpm_stepper_base {
  double Omega = 0;
  double* buf = nullptr;  // xs[4], zs[4], xw

  void advance(lpm_view vx, double* vzeta, lpm_view vvel, lpm_view fx,
               double* fzeta, lpm_view fvel, const double* farea,
               const uint8_t* fmask) {
    if (!ready) {
      setup(fmask);
      buf = static_cast<double*>(dalloc(sizeof(double) * size_t(T) * (4 * 3 + 4 + 3)));
    }
    lpm::Tg g = targets(vx, vzeta, vvel, nullptr, fx, fzeta, fvel, nullptr, farea);
    lpm::Pk k = packs();
    lpm::Rk4Buf b;
    for (int s = 0; s < 4; ++s) {
      b.xs[s] = buf + size_t(T) * 3 * s;
      b.zs[s] = buf + size_t(T) * 12 + size_t(T) * s;
    }
    b.xw = buf + size_t(T) * 16;
    lpm::Rk4Par P;
    P.dt = dt;
    P.Omega = Omega;
    P.fix_facevort3 = flags & LPM_STEP_FIX_FACEVORT3;
    P.reproject = flags & LPM_STEP_REPROJECT;
    P.c0 = c0();

    ff_prepare(g);
    std::vector<char> kk(sizeof(lpm::Tg) + sizeof(void*));
    std::memcpy(kk.data(), &g, sizeof(g));
    const void* fd = ff ? static_cast<const void*>(ff->d) : nullptr;
    std::memcpy(kk.data() + sizeof(g), &fd, sizeof(fd));
    const int64_t nb = (T + 255) / 256;
    run(kk, [&]() {
      if (T == 0) return;
      lpm::k_rk4_begin<<<nb, 256, 0, ctx->stream>>>(g, k, b, P);
      ctx->launches++;
      for (int s = 1; s <= 3; ++s) {
        nbody();
        lpm::k_rk4_stage<<<nb, 256, 0, ctx->stream>>>(g, k, b, P, s);
        ctx->launches++;
      }
      nbody();
      lpm::k_rk4_final<<<nb, 256, 0, ctx->stream>>>(g, k, b, P);
      ctx->launches++;
    });
  }
};

struct lpm_ic2d_rk2 : lpm_stepper_base {
  double cor = 0;
  double* buf = nullptr;

  void advance(lpm_view vx, double* vzeta, lpm_view vvel, double* vpsi,
               lpm_view fx, double* fzeta, lpm_view fvel, double* fpsi,
               const double* farea, const uint8_t* fmask) {
    if (!ready) {
      setup(fmask);
      buf = static_cast<double*>(dalloc(sizeof(double) * size_t(T) * (2 * ndim + 1)));
    }
    lpm::Tg g = targets(vx, vzeta, vvel, vpsi, fx, fzeta, fvel, fpsi, farea);
    lpm::Pk k = packs();
    lpm::Rk2Buf b;
    b.x1 = buf;
    b.z1 = buf + size_t(T) * ndim;
    b.xw = buf + size_t(T) * (ndim + 1);
    lpm::Rk2Par P;
    P.dt = dt;
    P.cor = cor;
    P.c0 = c0();
    P.sg = sgbuf;
    std::vector<char> kk(sizeof(lpm::Tg));
    std::memcpy(kk.data(), &g, sizeof(g));
    const int64_t nb = (T + 255) / 256;
    run(kk, [&]() {
      if (T == 0) return;
      lpm::k_rk2_begin<<<nb, 256, 0, ctx->stream>>>(g, k, b, P);
      ctx->launches++;
      // the stage-1 stream function is overwritten by the final evaluation
      // (as in Incompressible2DRK2::advance_timestep_impl), so it is not computed
      nbody(false);
      lpm::k_rk2_mid<<<nb, 256, 0, ctx->stream>>>(g, k, b, P);
      ctx->launches++;
      nbody();
      lpm::k_rk2_final<<<nb, 256, 0, ctx->stream>>>(g, k, b, P);
      ctx->launches++;
    });
  }
};

// ---------------------------------------------------------------------------
// C ABI of the steppers (the rest of the ABI is in capi.cu)
// ---------------------------------------------------------------------------
namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu
}

extern "C" {

int lpm_bve_rk4_create(lpm_context* ctx, lpm_bve_rk4** out, int64_t nverts,
                       int64_t nfaces, double dt, double Omega, double eps,
                       int precision, uint32_t flags) {
  try {
    if (!ctx || !out) return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_create: null argument");
    if (nverts < 0 || nfaces < 0 || nverts + nfaces > (int64_t(1) << 31) - 1)
      return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_create: sizes out of range");
    if (precision != LPM_FP64 && precision != LPM_FP32C && precision != LPM_FP64_CHORD &&
        precision != LPM_FP64_EXACT)
      return lpm::fail(LPM_ERR_ARG,
                       "lpm_bve_rk4_create: precision must be LPM_FP64, LPM_FP64_EXACT, "
                       "LPM_FP64_CHORD or LPM_FP32C");
    if (!std::isfinite(dt) || !std::isfinite(Omega) || !std::isfinite(eps) || eps < 0)
      return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_create: non-finite dt/Omega or bad eps");
    auto* st = new lpm_bve_rk4();
    st->ctx = ctx;
    st->ndim = 3;
    st->nv = nverts;
    st->nf = nfaces;
    st->dt = dt;
    st->Omega = Omega;
    st->eps = eps;
    st->precision = precision;
    st->flags = flags;
    st->form = eps == 0.0 ? lpm::FORM_BVE : lpm::FORM_SPHERE;
    st->skip_self = true;  // BVE face functors always skip i == j
    st->want_psi = false;
    *out = st;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_rk4_destroy(lpm_bve_rk4* st) {
  if (!st) return LPM_OK;
  lpm::DeviceGuard device_guard(st->ctx->device);
  st->free_all();
  delete st;
  return LPM_OK;
}

int lpm_bve_rk4_advance_timestep(lpm_bve_rk4* st, lpm_view vx, double* vzeta,
                                 lpm_view vvel, lpm_view fx, double* fzeta,
                                 lpm_view fvel, const double* farea,
                                 const uint8_t* fmask) {
  try {
    if (!st) return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_advance_timestep: null stepper");
    if ((st->nv > 0 && (!vx.p || !vzeta || !vvel.p)) ||
        (st->nf > 0 && (!fx.p || !fzeta || !fvel.p || !farea || !fmask)))
      return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_advance_timestep: null array");
    lpm::DeviceGuard device_guard(st->ctx->device);
    st->advance(vx, vzeta, vvel, fx, fzeta, fvel, farea, fmask);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ic2d_rk2_create(lpm_context* ctx, lpm_ic2d_rk2** out, int ndim,
                        int64_t nverts, int64_t nfaces, double dt, double eps,
                        double cor, int precision, uint32_t flags) {
  try {
    if (!ctx || !out) return lpm::fail(LPM_ERR_ARG, "lpm_ic2d_rk2_create: null argument");
    if (ndim != LPM_SPHERE && ndim != LPM_PLANE)
      return lpm::fail(LPM_ERR_ARG, "lpm_ic2d_rk2_create: ndim must be 2 or 3");
    if (nverts < 0 || nfaces < 0 || nverts + nfaces > (int64_t(1) << 31) - 1)
      return lpm::fail(LPM_ERR_ARG, "lpm_ic2d_rk2_create: sizes out of range");
    if (precision != LPM_FP64 && precision != LPM_FP32C && precision != LPM_FP64_CHORD &&
        precision != LPM_FP64_EXACT)
      return lpm::fail(LPM_ERR_ARG, "lpm_ic2d_rk2_create: bad precision");
    if (!std::isfinite(dt) || !std::isfinite(cor) || !std::isfinite(eps) || eps < 0)
      return lpm::fail(LPM_ERR_ARG, "lpm_ic2d_rk2_create: non-finite dt/cor or bad eps");
    auto* st = new lpm_ic2d_rk2();
    st->ctx = ctx;
    st->ndim = ndim;
    st->nv = nverts;
    st->nf = nfaces;
    st->dt = dt;
    st->eps = eps;
    st->cor = cor;
    st->precision = precision;
    st->flags = flags;
    st->form = ndim == 3 ? lpm::FORM_SPHERE : lpm::FORM_PLANE;
    // Incompressible2DActiveSums: skip i == j only when eps is zero (:235)
    st->skip_self = (std::fabs(eps) < 2.220446049250313e-16) ||
                    (flags & LPM_STEP_SKIP_SELF_ALWAYS);
    st->want_psi = true;
    *out = st;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ic2d_rk2_destroy(lpm_ic2d_rk2* st) {
  if (!st) return LPM_OK;
  lpm::DeviceGuard device_guard(st->ctx->device);
  st->free_all();
  delete st;
  return LPM_OK;
}

int lpm_ic2d_rk2_advance_timestep(lpm_ic2d_rk2* st, lpm_view vx,
                                  double* vzeta, lpm_view vvel, double* vpsi,
                                  lpm_view fx, double* fzeta, lpm_view fvel,
                                  double* fpsi, const double* farea,
                                  const uint8_t* fmask) {
  try {
    if (!st) return lpm::fail(LPM_ERR_ARG, "lpm_ic2d_rk2_advance_timestep: null stepper");
    if ((st->nv > 0 && (!vx.p || !vzeta || !vvel.p)) ||
        (st->nf > 0 && (!fx.p || !fzeta || !fvel.p || !farea || !fmask)))
      return lpm::fail(LPM_ERR_ARG, "lpm_ic2d_rk2_advance_timestep: null array");
    lpm::DeviceGuard device_guard(st->ctx->device);
    st->advance(vx, vzeta, vvel, vpsi, fx, fzeta, fvel, fpsi, farea, fmask);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_rk4_set_farfield(lpm_bve_rk4* st, lpm_farfield* ff, int rebuild_every) {
  if (!st) return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_set_farfield: null stepper");
  if (ff && st->precision != LPM_FP64_CHORD)
    return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_set_farfield: the stepper must use LPM_FP64_CHORD");
  if (ff && ff->ctx != st->ctx)
    return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_set_farfield: far field and stepper contexts differ");
  if (rebuild_every < 0) return lpm::fail(LPM_ERR_ARG, "lpm_bve_rk4_set_farfield: rebuild_every < 0");
  st->ff = ff;
  st->ff_every = rebuild_every;
  st->ff_steps = 0;
  return LPM_OK;
}

int lpm_bve_rk4_nbody_time(lpm_bve_rk4* st, double* ms, int64_t* launches) {
  try {
    if (!st || !ms || !launches) return lpm::fail(LPM_ERR_ARG, "null argument");
    lpm::DeviceGuard device_guard(st->ctx->device);
    st->nbody_time(ms, launches);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_bve_rk4_kernel_shape(lpm_bve_rk4* st, int* threads, int* targets_per_thread,
                             int* min_ctas_per_sm) {
  if (!st || !threads || !targets_per_thread || !min_ctas_per_sm)
    return lpm::fail(LPM_ERR_ARG, "null argument");
  if (!st->ready)
    return lpm::fail(LPM_ERR_STATE, "lpm_bve_rk4_kernel_shape: no step taken yet");
  if (st->precision == LPM_FP32C) {
    const lpm::F32Shape& k = lpm::kF32Shapes[st->plan.shape];
    *threads = k.nt;
    *targets_per_thread = k.r;
    *min_ctas_per_sm = k.minb;
  } else {
    *threads = lpm::F64_NT;
    *targets_per_thread = lpm::F64_R;
    *min_ctas_per_sm = 0;
  }
  return LPM_OK;
}

int lpm_ic2d_rk2_nbody_time(lpm_ic2d_rk2* st, double* ms, int64_t* launches) {
  try {
    if (!st || !ms || !launches) return lpm::fail(LPM_ERR_ARG, "null argument");
    lpm::DeviceGuard device_guard(st->ctx->device);
    st->nbody_time(ms, launches);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

}  // extern "C"

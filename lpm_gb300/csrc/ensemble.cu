// ensemble.cu -- many independent BVE sphere problems of uneven size advanced
// together: every evaluation is ONE N-body launch over a work list
// of (problem, target block, source chunk) items, and a whole RK4 step (four
// evaluations plus the fused stage epilogues) is captured once into a CUDA
// graph and replayed.
//
// Layout: problem-major.  Problem p owns [toff[p], toff[p] + tpad[p]) of the
// packed targets (its vertices, then its face targets, padded to a whole
// number of target blocks; padding entries are skipped), [soff[p], soff[p] +
// spad[p]) of the packed sources (its unmasked faces, zero-padded to a whole
// number of tiles) and its own block of chunk partials.  The work list is
// sorted by decreasing chunk length, so the persistent CTAs drain it
// longest-first and the tail stays short.  The chunk length and the FP32
// kernel shape (threads x targets per thread, the kF32Shapes of the
// single-problem kernel) and the launch form (persistent CTAs draining the
// list, or one CTA per item launched longest first) are chosen by an
// autotuner that times one evaluation per candidate at set-up: chunk
// lengths with the default shape in the persistent form, then every shape in
// both forms at the best length, keeping the persistent form unless the other
// is more than 1 % faster.  A target's sums do not depend on the
// shape (each target is summed by one thread in source order), so only the
// chunk length changes results in the last bits.
//
// Only the chord-form velocity is evaluated (LPM_FP32C or LPM_FP64_CHORD);
// the reference-arithmetic FP64 path runs one problem at a time through
// lpm_bve_rk4.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "lpm_host.hpp"
#include "nbody.cuh"
#include "stage.cuh"

namespace lpm {
namespace {

// One work item of the persistent kernel, compiled out of line: inlined into
// the item loop the pair loop took ~3 more ALU instructions per pair (0.79 of
// the FP32 peak against 0.95 for the same body launched one CTA per item);
// out of line it compiles like the per-item kernel.
template <typename T, int R, int NT, int TILE>
__device__ __noinline__ bool ens_item(int it, const int4* __restrict__ items,
                                      const typename Vec4<T>::type* __restrict__ tgt,
                                      const typename SrcRec<T>::type* __restrict__ src,
                                      const int64_t* ptoff, const int64_t* ptpad,
                                      const int64_t* psoff, const int64_t* pspad,
                                      const int64_t* ppart, int chunk_len, T c0,
                                      double* __restrict__ part, int* err,
                                      typename SrcRec<T>::type* sbuf, uint64_t* sbar,
                                      unsigned& g0) {
  using V4 = typename Vec4<T>::type;
  using Rec = typename SrcRec<T>::type;
  constexpr int NC = 3;
  const int tid = threadIdx.x;
  const int4 w = items[it];  // (problem, target block, chunk, -)
  const int p = w.x;
  const int64_t tl = (int64_t)w.y * (NT * R);
  const int64_t sl = (int64_t)w.z * chunk_len;
  int64_t slen = pspad[p] - sl;
  if (slen > chunk_len) slen = chunk_len;
  TilePipe<Rec, TILE> pipe{sbuf, sbar, src + psoff[p] + sl, int(slen / TILE)};
  pipe.g0 = g0;
  pipe.prefetch();
  T tx[R], ty[R], tz[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const V4 t = tgt[ptoff[p] + tl + r * NT + tid];
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
  if (!chord_chunk<T, 3, true, false, false, R, TILE>(pipe, tx, ty, tz, S, C, c0, err))
    return false;
  g0 += unsigned(pipe.ntiles);
  const int64_t tp = ptpad[p];
  double* out = part + ppart[p] + (int64_t)w.z * NC * tp + tl;
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r) out[k * tp + r * NT + tid] = (double)S[k][r] + (double)C[k][r];
  return true;
}

// Persistent chord-form velocity kernel over the work list.
template <typename T, int R, int NT, int TILE, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    ens_nbody(const int4* __restrict__ items, int nitems, int* counter,
              const typename Vec4<T>::type* __restrict__ tgt,
              const typename SrcRec<T>::type* __restrict__ src, const int64_t* ptoff,
              const int64_t* ptpad, const int64_t* psoff, const int64_t* pspad,
              const int64_t* ppart, int chunk_len, T c0, double* __restrict__ part,
              int* err) {
  using Rec = typename SrcRec<T>::type;
  __shared__ __align__(128) Rec sbuf[2 * TILE];
  __shared__ __align__(8) uint64_t sbar[2];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  {
    TilePipe<Rec, TILE> init_pipe{sbuf, sbar, src, 0};
    init_pipe.init();
  }
  unsigned g0 = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= nitems) return;
    if (!ens_item<T, R, NT, TILE>(it, items, tgt, src, ptoff, ptpad, psoff, pspad, ppart,
                                  chunk_len, c0, part, err, sbuf, sbar, g0))
      return;
  }
}

// The same work items with one CTA each (item = blockIdx.x): the items are
// ordered longest first, so the hardware's CTA scheduler drains them in that
// order as resident slots free up.  The body is the persistent kernel's
// without the item loop; the sums are the same bit for bit.
template <typename T, int R, int NT, int TILE, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    ens_nbody_items(const int4* __restrict__ items,
                    const typename Vec4<T>::type* __restrict__ tgt,
                    const typename SrcRec<T>::type* __restrict__ src, const int64_t* ptoff,
                    const int64_t* ptpad, const int64_t* psoff, const int64_t* pspad,
                    const int64_t* ppart, int chunk_len, T c0, double* __restrict__ part,
                    int* err) {
  using V4 = typename Vec4<T>::type;
  using Rec = typename SrcRec<T>::type;
  constexpr int NC = 3;
  __shared__ __align__(128) Rec sbuf[2 * TILE];
  __shared__ __align__(8) uint64_t sbar[2];
  const int tid = threadIdx.x;
  const int4 w = items[blockIdx.x];  // (problem, target block, chunk, -)
  const int p = w.x;
  const int64_t tl = (int64_t)w.y * (NT * R);
  const int64_t sl = (int64_t)w.z * chunk_len;
  int64_t slen = pspad[p] - sl;
  if (slen > chunk_len) slen = chunk_len;
  TilePipe<Rec, TILE> pipe{sbuf, sbar, src + psoff[p] + sl, int(slen / TILE)};
  pipe.start();
  T tx[R], ty[R], tz[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const V4 t = tgt[ptoff[p] + tl + r * NT + tid];
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
  if (!chord_chunk<T, 3, true, false, false, R, TILE>(pipe, tx, ty, tz, S, C, c0, err)) return;
  const int64_t tp = ptpad[p];
  double* out = part + ppart[p] + (int64_t)w.z * NC * tp + tl;
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r) out[k * tp + r * NT + tid] = (double)S[k][r] + (double)C[k][r];
}

// Packs the current state (positions, vorticity) for an evaluation and
// records the evaluation positions.
template <class TG, class PK>
__global__ void k_ens_pack_state(TG g, PK k, double* xw) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.T || !g.valid(t)) return;
  double p[3];
  for (int c = 0; c < 3; ++c) {
    p[c] = g.x(t, c);
    xw[c * g.T + t] = p[c];
  }
  pack(g, k, t, p, g.face(t) ? g.zeta(t) : 0.0);  // vertex vorticity is not a source
}

}  // namespace
}  // namespace lpm

namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu
}

struct lpm_ensemble {
  lpm_context* ctx = nullptr;
  int nprob = 0;
  double dt = 0, Omega = 0, eps = 0;
  int precision = LPM_FP32C;
  uint32_t flags = 0;
  int64_t NV = 0, NF = 0, T = 0, S = 0;
  std::vector<int64_t> nv, nf, toff, tpad, soff, spad;
  int chunk_len = 0;
  int64_t nitems = 0;
  std::vector<void*> allocs;
  // device tables
  int *tix = nullptr, *tprob = nullptr, *slot2src = nullptr, *counter = nullptr;
  int64_t *d_toff = nullptr, *d_tpad = nullptr, *d_soff = nullptr, *d_spad = nullptr,
          *d_ppart = nullptr;
  int* d_pchunks = nullptr;
  int4* items = nullptr;
  void *tgt = nullptr, *src = nullptr;
  double* part = nullptr;
  double* buf = nullptr;  // xs[4] (3T each), zs[4] (T each), xw (3T)
  int shape = 0;         // FP32 kernel shape (index into kF32Shapes)
  bool persistent = true;  // launch form: persistent CTAs or one CTA per item
  int occ_shape[lpm::kNumF32Shapes] = {};  // resident CTAs per SM, per shape
  // graph
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<char> key;
  int64_t graph_kernels = 0;
  std::vector<cudaEvent_t> timers;

  bool f32() const { return precision == LPM_FP32C; }
  // target padding unit (every FP32 shape divides F32_TB)
  int tb() const { return f32() ? lpm::F32_TB : lpm::F64_NT * lpm::F64_R; }
  // targets per CTA of the kernel in use
  int cta_targets() const {
    return f32() ? lpm::kF32Shapes[shape].nt * lpm::kF32Shapes[shape].r
                 : lpm::F64_NT * lpm::F64_R;
  }
  int tile() const { return f32() ? lpm::F32_TILE : lpm::F64_TILE; }

  void* dalloc(size_t bytes) {
    void* p = nullptr;
    LPM_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
    allocs.push_back(p);
    return p;
  }
  template <typename V>
  void* upload(const std::vector<V>& h) {
    void* d = dalloc(sizeof(V) * h.size());
    if (!h.empty())
      LPM_CUDA(cudaMemcpy(d, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice));
    return d;
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
    for (void* p : plan_allocs) cudaFree(p);
    plan_allocs.clear();
  }

  void setup(const std::vector<uint8_t>& mask) {
    const bool skip_masked = flags & LPM_STEP_SKIP_MASKED_TARGETS;
    const int TB = tb(), TL = tile();
    toff.resize(nprob);
    tpad.resize(nprob);
    soff.resize(nprob);
    spad.resize(nprob);
    std::vector<int> h_tix, h_tprob, h_slot2src(NF, -1);
    int64_t vbase = 0, fbase = 0;
    T = 0;
    S = 0;
    for (int p = 0; p < nprob; ++p) {
      int64_t nsrc = 0;
      std::vector<int> faces;
      for (int64_t s = 0; s < nf[p]; ++s) {
        const bool leaf = !mask[fbase + s];
        if (leaf) h_slot2src[fbase + s] = int(S + nsrc++);
        if (leaf || !skip_masked) faces.push_back(int(fbase + s));
      }
      const int64_t tp = nv[p] + int64_t(faces.size());
      toff[p] = T;
      tpad[p] = std::max<int64_t>(TB, (tp + TB - 1) / TB * TB);
      soff[p] = S;
      spad[p] = std::max<int64_t>(TL, (nsrc + TL - 1) / TL * TL);
      for (int64_t i = 0; i < nv[p]; ++i) h_tix.push_back(int(vbase + i));
      for (int f : faces) h_tix.push_back(-f - 1);
      for (int64_t i = tp; i < tpad[p]; ++i) h_tix.push_back(lpm::kPadTarget);
      for (int64_t i = 0; i < tpad[p]; ++i) h_tprob.push_back(p);
      T += tpad[p];
      S += spad[p];
      vbase += nv[p];
      fbase += nf[p];
    }
    tix = static_cast<int*>(upload(h_tix));
    tprob = static_cast<int*>(upload(h_tprob));
    slot2src = static_cast<int*>(upload(h_slot2src));
    d_toff = static_cast<int64_t*>(upload(toff));
    d_tpad = static_cast<int64_t*>(upload(tpad));
    d_soff = static_cast<int64_t*>(upload(soff));
    d_spad = static_cast<int64_t*>(upload(spad));
    const size_t rec = f32() ? 16 : 32;
    tgt = dalloc(rec * T);
    src = dalloc(32 * S);  // SrcF32 / double4_16a
    LPM_CUDA(cudaMemset(tgt, 0, rec * T));
    LPM_CUDA(cudaMemset(src, 0, 32 * S));
    counter = static_cast<int*>(dalloc(sizeof(int)));
    buf = static_cast<double*>(dalloc(sizeof(double) * size_t(T) * 19));
    if (f32()) {
      static_assert(lpm::kF32Shapes[0].nt == 256 && lpm::kF32Shapes[0].r == 4 &&
                        lpm::kF32Shapes[1].nt == 256 && lpm::kF32Shapes[1].r == 4 &&
                        lpm::kF32Shapes[2].nt == 128 && lpm::kF32Shapes[2].r == 8 &&
                        lpm::kF32Shapes[3].nt == 256 && lpm::kF32Shapes[3].r == 2 &&
                        lpm::kF32Shapes[4].nt == 128 && lpm::kF32Shapes[4].r == 8 &&
                        lpm::kF32Shapes[5].nt == 256 && lpm::kF32Shapes[5].r == 4 &&
                        lpm::kNumF32Shapes == 6,
                    "ensemble launch table out of sync with kF32Shapes");
      occupancy(0, lpm::ens_nbody<float, 4, 256, lpm::F32_TILE, 3>, 256);
      occupancy(1, lpm::ens_nbody<float, 4, 256, lpm::F32_TILE, 4>, 256);
      occupancy(2, lpm::ens_nbody<float, 8, 128, lpm::F32_TILE, 4>, 128);
      occupancy(3, lpm::ens_nbody<float, 2, 256, lpm::F32_TILE, 5>, 256);
      occupancy(4, lpm::ens_nbody<float, 8, 128, lpm::F32_TILE, 3>, 128);
      occupancy(5, lpm::ens_nbody<float, 4, 256, lpm::F32_TILE, 2>, 256);
    } else {
      occupancy(0, lpm::ens_nbody<double, lpm::F64_R, lpm::F64_NT, lpm::F64_TILE, 1>,
                lpm::F64_NT);
    }
    LPM_CUDA(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
  }

  template <class K>
  void occupancy(int k, K kernel, int nt) {
    int v = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, nt, 0);
    occ_shape[k] = std::max(v, 1);
  }

  // Work list and partial layout for a chunk length (in sources) and the
  // current kernel shape: one item per (problem, CTA target block, chunk).
  void plan(int chunk) {
    chunk_len = chunk;
    const int TB = cta_targets();
    std::vector<int64_t> ppart(nprob);
    std::vector<int> pch(nprob);
    struct It {
      int p, tb, c;
      int64_t len;
    };
    std::vector<It> its;
    int64_t pb = 0;
    for (int p = 0; p < nprob; ++p) {
      pch[p] = int((spad[p] + chunk - 1) / chunk);
      ppart[p] = pb;
      pb += int64_t(3) * pch[p] * tpad[p];
      for (int c = 0; c < pch[p]; ++c) {
        const int64_t len = std::min<int64_t>(chunk, spad[p] - int64_t(c) * chunk);
        for (int64_t b = 0; b < tpad[p] / TB; ++b) its.push_back({p, int(b), c, len});
      }
    }
    std::stable_sort(its.begin(), its.end(), [](const It& a, const It& b) { return a.len > b.len; });
    std::vector<int4> h(its.size());
    for (size_t i = 0; i < its.size(); ++i) h[i] = make_int4(its[i].p, its[i].tb, its[i].c, 0);
    nitems = int64_t(h.size());
    // replace the previous plan's tables (plans change during autotuning only)
    for (void* q : plan_allocs) cudaFree(q);
    plan_allocs.clear();
    const size_t keep = allocs.size();
    items = static_cast<int4*>(upload(h));
    d_ppart = static_cast<int64_t*>(upload(ppart));
    d_pchunks = static_cast<int*>(upload(pch));
    part = static_cast<double*>(dalloc(sizeof(double) * size_t(pb)));
    plan_allocs.assign(allocs.begin() + keep, allocs.end());
    allocs.resize(keep);
  }
  std::vector<void*> plan_allocs;

  lpm::EnsTg targets(lpm_view vx, double* vzeta, lpm_view vvel, lpm_view fx,
                     double* fzeta, lpm_view fvel, const double* farea) const {
    lpm::EnsTg g;
    g.ndim = 3;
    g.T = T;
    g.tix = tix;
    g.slot2src = slot2src;
    g.vx = lpm::to_view(vx);
    g.fx = lpm::to_view(fx);
    g.vvel = lpm::to_view(vvel);
    g.fvel = lpm::to_view(fvel);
    g.vzeta = vzeta;
    g.fzeta = fzeta;
    g.vpsi = nullptr;
    g.fpsi = nullptr;
    g.farea = farea;
    return g;
  }
  lpm::EnsPk packs() const {
    lpm::EnsPk k;
    k.mode = lpm::mode_of(precision);
    k.form = lpm::FORM_SPHERE;
    k.skip_self = true;
    k.tgt = tgt;
    k.tself = nullptr;
    k.src = src;
    k.part = part;
    k.tprob = tprob;
    k.pbase_ = d_ppart;
    k.pchunks = d_pchunks;
    k.ptpad = d_tpad;
    k.ptoff = d_toff;
    return k;
  }
  double c0() const {
    return f32() ? double(lpm::f32_c0(3, eps)) : lpm::chord_c0(3, eps);
  }

  void nbody() {
    lpm_context& c = *ctx;
    LPM_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), c.stream));
    const int grid = c.num_sms * occ_shape[f32() ? shape : 0];
    cudaEvent_t e[2];
    const bool timed = flags & LPM_STEP_TIME_NBODY;
    if (timed) {
      LPM_CUDA(cudaEventCreate(&e[0]));
      LPM_CUDA(cudaEventCreate(&e[1]));
      LPM_CUDA(cudaEventRecord(e[0], c.stream));
    }
    if (f32()) {
      switch (shape) {
        case 1:
          launch_f32<4, 256, 4>(grid);
          break;
        case 2:
          launch_f32<8, 128, 4>(grid);
          break;
        case 3:
          launch_f32<2, 256, 5>(grid);
          break;
        case 4:
          launch_f32<8, 128, 3>(grid);
          break;
        case 5:
          launch_f32<4, 256, 2>(grid);
          break;
        default:
          launch_f32<4, 256, 3>(grid);
      }
    } else {
      lpm::ens_nbody<double, lpm::F64_R, lpm::F64_NT, lpm::F64_TILE, 1>
          <<<grid, lpm::F64_NT, 0, c.stream>>>(
              items, int(nitems), counter, static_cast<const double4_16a*>(tgt),
              static_cast<const double4_16a*>(src), d_toff, d_tpad, d_soff, d_spad, d_ppart,
              chunk_len, c0(), part, c.d_err);
    }
    c.launches++;
    if (timed) {
      LPM_CUDA(cudaEventRecord(e[1], c.stream));
      timers.push_back(e[0]);
      timers.push_back(e[1]);
    }
    LPM_CUDA(cudaGetLastError());
  }

  template <int R, int NT, int MINB>
  void launch_f32(int grid) {
    if (!persistent) {
      lpm::ens_nbody_items<float, R, NT, lpm::F32_TILE, MINB>
          <<<unsigned(nitems), NT, 0, ctx->stream>>>(
              items, static_cast<const float4*>(tgt), static_cast<const lpm::SrcF32*>(src),
              d_toff, d_tpad, d_soff, d_spad, d_ppart, chunk_len, float(c0()), part, ctx->d_err);
      return;
    }
    lpm::ens_nbody<float, R, NT, lpm::F32_TILE, MINB><<<grid, NT, 0, ctx->stream>>>(
        items, int(nitems), counter, static_cast<const float4*>(tgt),
        static_cast<const lpm::SrcF32*>(src), d_toff, d_tpad, d_soff, d_spad, d_ppart,
        chunk_len, float(c0()), part, ctx->d_err);
  }

  // One evaluation of the current state's velocities into vvel / fvel.
  void velocity(const lpm::EnsTg& g) {
    lpm::EnsPk k = packs();
    lpm::Rk4Buf b = bufs();
    lpm::Rk4Par P = params();
    const int64_t nb = (T + 255) / 256;
    lpm::k_ens_pack_state<<<nb, 256, 0, ctx->stream>>>(g, k, b.xw);
    ctx->launches++;
    nbody();
    lpm::k_rk4_final<<<nb, 256, 0, ctx->stream>>>(g, k, b, P);
    ctx->launches++;
    LPM_CUDA(cudaGetLastError());
  }

  lpm::Rk4Buf bufs() const {
    lpm::Rk4Buf b;
    for (int s = 0; s < 4; ++s) {
      b.xs[s] = buf + size_t(T) * 3 * s;
      b.zs[s] = buf + size_t(T) * 12 + size_t(T) * s;
    }
    b.xw = buf + size_t(T) * 16;
    return b;
  }
  lpm::Rk4Par params() const {
    lpm::Rk4Par P;
    P.dt = dt;
    P.Omega = Omega;
    P.fix_facevort3 = flags & LPM_STEP_FIX_FACEVORT3;
    P.reproject = flags & LPM_STEP_REPROJECT;
    P.c0 = c0();
    return P;
  }

  void step_body(const lpm::EnsTg& g) {
    lpm::EnsPk k = packs();
    lpm::Rk4Buf b = bufs();
    lpm::Rk4Par P = params();
    const int64_t nb = (T + 255) / 256;
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
    LPM_CUDA(cudaGetLastError());
  }

  void advance(const lpm::EnsTg& g) {
    lpm_context& c = *ctx;
    if (flags & (LPM_STEP_NO_GRAPH | LPM_STEP_TIME_NBODY)) {
      step_body(g);
      return;
    }
    std::vector<char> kk(sizeof(g));
    std::memcpy(kk.data(), &g, sizeof(g));
    if (!exec || kk != key) {
      if (exec) cudaGraphExecDestroy(exec);
      exec = nullptr;
      cudaStream_t user = c.stream;
      const int64_t before = c.launches;
      LPM_CUDA(cudaStreamSynchronize(user));
      c.stream = cap_stream;
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        try {
          step_body(g);
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
      key = kk;
    }
    LPM_CUDA(cudaGraphLaunch(exec, c.stream));
    c.launches += graph_kernels;
  }

  // Times one evaluation per candidate chunk length and keeps the fastest.
  void autotune(const lpm::EnsTg& g) {
    const int TL = tile();
    const int64_t smax = *std::max_element(spad.begin(), spad.end());
    std::vector<int> cands;
    for (int tiles : {4, 8, 16, 32, 64}) {
      const int64_t len = int64_t(tiles) * TL;
      if (len <= std::max<int64_t>(smax, TL)) cands.push_back(int(len));
    }
    if (cands.empty()) cands.push_back(TL);
    lpm::EnsPk k = packs();
    lpm::Rk4Buf b = bufs();
    const int64_t nb = (T + 255) / 256;
    lpm::k_ens_pack_state<<<nb, 256, 0, ctx->stream>>>(g, k, b.xw);
    ctx->launches++;
    float best = 1e30f;
    int best_len = cands.front();
    cudaEvent_t e0, e1;
    LPM_CUDA(cudaEventCreate(&e0));
    LPM_CUDA(cudaEventCreate(&e1));
    const uint32_t saved = flags;
    flags &= ~LPM_STEP_TIME_NBODY;
    auto time_plan = [&]() {
      nbody();  // warm
      LPM_CUDA(cudaEventRecord(e0, ctx->stream));
      nbody();
      LPM_CUDA(cudaEventRecord(e1, ctx->stream));
      LPM_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      LPM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms;
    };
    // chunk length with the default shape and the persistent form
    shape = 0;
    persistent = true;
    for (int len : cands) {
      plan(len);
      const float ms = time_plan();
      if (ms < best) {
        best = ms;
        best_len = len;
      }
    }
    // kernel shape and launch form at that chunk length; the one-CTA-per-item
    // form is taken only when it is more than 1 % faster (with the persistent
    // kernel's item body out of line the two measure within a few tenths of a
    // percent)
    int best_shape = 0;
    bool best_persistent = true;
    float best_raw = best;
    if (f32()) {
      for (int form = 0; form < 2; ++form)
        for (int k = 0; k < lpm::kNumF32Shapes; ++k) {
          if (form == 0 && k == 0) continue;  // timed above
          shape = k;
          persistent = form == 0;
          plan(best_len);
          const float raw = time_plan();
          const float ms = raw * (persistent ? 1.0f : 1.01f);
          if (ms < best) {
            best = ms;
            best_raw = raw;
            best_shape = k;
            best_persistent = persistent;
          }
        }
    }
    flags = saved;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    shape = best_shape;
    persistent = best_persistent;
    plan(best_len);
    tuned_ms = best_raw;
  }
  float tuned_ms = 0;
};

extern "C" {

int lpm_ensemble_create(lpm_context* ctx, lpm_ensemble** out, int nproblems,
                        const int64_t* nverts, const int64_t* nfaces,
                        const uint8_t* fmask, double dt, double Omega, double eps,
                        int precision, uint32_t flags) {
  try {
    if (!ctx || !out || !nverts || !nfaces || nproblems <= 0)
      return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_create: null argument or no problems");
    if (precision != LPM_FP32C && precision != LPM_FP64_CHORD)
      return lpm::fail(LPM_ERR_ARG,
                       "lpm_ensemble_create: precision must be LPM_FP32C or LPM_FP64_CHORD");
    if (!std::isfinite(dt) || !std::isfinite(Omega) || !std::isfinite(eps) || eps < 0)
      return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_create: non-finite dt/Omega or bad eps");
    auto* e = new lpm_ensemble();
    e->ctx = ctx;
    e->nprob = nproblems;
    e->dt = dt;
    e->Omega = Omega;
    e->eps = eps;
    e->precision = precision;
    e->flags = flags;
    for (int p = 0; p < nproblems; ++p) {
      if (nverts[p] < 0 || nfaces[p] <= 0) {
        delete e;
        return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_create: every problem needs face slots");
      }
      e->nv.push_back(nverts[p]);
      e->nf.push_back(nfaces[p]);
      e->NV += nverts[p];
      e->NF += nfaces[p];
    }
    if (e->NV + e->NF > (int64_t(1) << 30)) {
      delete e;
      return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_create: too many particles");
    }
    if (!fmask) {
      delete e;
      return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_create: null mask");
    }
    lpm::DeviceGuard device_guard(ctx->device);
    std::vector<uint8_t> hmask(e->NF);
    LPM_CUDA(cudaMemcpy(hmask.data(), fmask, e->NF, cudaMemcpyDeviceToHost));
    try {
      e->setup(hmask);
    } catch (...) {
      e->free_all();
      delete e;
      throw;
    }
    *out = e;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ensemble_destroy(lpm_ensemble* e) {
  if (!e) return LPM_OK;
  lpm::DeviceGuard device_guard(e->ctx->device);
  e->free_all();
  delete e;
  return LPM_OK;
}

int lpm_ensemble_velocity(lpm_ensemble* e, lpm_view vx, lpm_view vvel, lpm_view fx,
                          const double* fzeta, lpm_view fvel, const double* farea) {
  try {
    if (!e || !vx.p || !vvel.p || !fx.p || !fzeta || !fvel.p || !farea)
      return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_velocity: null argument");
    lpm::DeviceGuard device_guard(e->ctx->device);
    lpm::EnsTg g = e->targets(vx, nullptr, vvel, fx, const_cast<double*>(fzeta), fvel, farea);
    // vertex vorticity is not read by an evaluation
    if (e->chunk_len == 0) e->autotune(g);
    e->velocity(g);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ensemble_advance_timestep(lpm_ensemble* e, lpm_view vx, double* vzeta,
                                  lpm_view vvel, lpm_view fx, double* fzeta,
                                  lpm_view fvel, const double* farea) {
  try {
    if (!e || !vx.p || !vzeta || !vvel.p || !fx.p || !fzeta || !fvel.p || !farea)
      return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_advance_timestep: null argument");
    lpm::DeviceGuard device_guard(e->ctx->device);
    lpm::EnsTg g = e->targets(vx, vzeta, vvel, fx, fzeta, fvel, farea);
    if (e->chunk_len == 0) e->autotune(g);
    e->advance(g);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ensemble_info(lpm_ensemble* e, int64_t* chunk_len, int64_t* items,
                      int64_t* targets) {
  if (!e || !chunk_len || !items || !targets) return lpm::fail(LPM_ERR_ARG, "null argument");
  *chunk_len = e->chunk_len;
  *items = e->nitems;
  *targets = e->T;
  return LPM_OK;
}

int lpm_ensemble_shape(lpm_ensemble* e, int* threads, int* targets_per_thread,
                       int* persistent) {
  if (!e || !threads || !targets_per_thread) return lpm::fail(LPM_ERR_ARG, "null argument");
  if (persistent) *persistent = e->persistent ? 1 : 0;
  if (e->f32()) {
    *threads = lpm::kF32Shapes[e->shape].nt;
    *targets_per_thread = lpm::kF32Shapes[e->shape].r;
  } else {
    *threads = lpm::F64_NT;
    *targets_per_thread = lpm::F64_R;
  }
  return LPM_OK;
}

int lpm_ensemble_set_kernel(lpm_ensemble* e, int shape, int persistent) {
  if (!e || shape < 0 || shape >= lpm::kNumF32Shapes)
    return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_set_kernel: bad argument");
  if (e->chunk_len != 0)
    return lpm::fail(LPM_ERR_STATE, "lpm_ensemble_set_kernel: plan already chosen");
  e->shape = e->f32() ? shape : 0;
  e->persistent = e->f32() ? persistent != 0 : true;
  return LPM_OK;
}

int lpm_ensemble_set_chunk_len(lpm_ensemble* e, int64_t chunk_len) {
  try {
    if (!e || chunk_len <= 0 || chunk_len > (int64_t(1) << 30))
      return lpm::fail(LPM_ERR_ARG, "lpm_ensemble_set_chunk_len: bad argument");
    if (e->chunk_len != 0)
      return lpm::fail(LPM_ERR_STATE, "lpm_ensemble_set_chunk_len: plan already chosen");
    lpm::DeviceGuard device_guard(e->ctx->device);
    const int64_t tl = e->tile();
    e->plan(int((chunk_len + tl - 1) / tl * tl));
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_ensemble_nbody_time(lpm_ensemble* e, double* ms, int64_t* launches) {
  try {
    if (!e || !ms || !launches) return lpm::fail(LPM_ERR_ARG, "null argument");
    LPM_CUDA(cudaStreamSynchronize(e->ctx->stream));
    double tot = 0;
    for (size_t i = 0; i + 1 < e->timers.size(); i += 2) {
      float m = 0;
      LPM_CUDA(cudaEventElapsedTime(&m, e->timers[i], e->timers[i + 1]));
      tot += m;
    }
    *ms = tot;
    *launches = int64_t(e->timers.size() / 2);
    for (cudaEvent_t ev : e->timers) cudaEventDestroy(ev);
    e->timers.clear();
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

}  // extern "C"

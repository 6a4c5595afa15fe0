// ffapi.cu -- extern "C" entry points of the octree far field with the learned
// correction (include/lpm_gb300.h, "Octree far field").
#include <cmath>
#include <string>
#include <vector>

#include "farfield_dev.cuh"
#include "lpm_host.hpp"
#include "nbody.cuh"

namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu
}  // namespace lpm

namespace {

using lpm::fail;

__global__ void k_ff_pack_src(lpm::View fx, const double* __restrict__ zeta,
                              const double* __restrict__ area, const int* __restrict__ src2slot,
                              int64_t ns, double4_16a* __restrict__ src) {
  const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= ns) return;
  const int64_t s = src2slot[k];
  src[k] = make_double4_16a(fx(s, 0), fx(s, 1), fx(s, 2), zeta[s] * area[s]);
}

__global__ void k_ff_pack_tgt(lpm::View x, int64_t n, double4_16a* __restrict__ tgt) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  tgt[i] = make_double4_16a(x(i, 0), x(i, 1), x(i, 2), 0.0);
}

// u = -(1/2pi) w cross x
__global__ void k_ff_velocity(const double* __restrict__ w, int64_t n, lpm::View x, lpm::View u) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const double w0 = w[i], w1 = w[n + i], w2 = w[2 * n + i];
  const double x0 = x(i, 0), x1 = x(i, 1), x2 = x(i, 2);
  const double k = -1.0 / lpm::kTWOPI;
  u(i, 0) = k * (w1 * x2 - w2 * x1);
  u(i, 1) = k * (w2 * x0 - w0 * x2);
  u(i, 2) = k * (w0 * x1 - w1 * x0);
}

__global__ void k_ff_zero(int64_t n, lpm::View u) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  u(i, 0) = 0.0;
  u(i, 1) = 0.0;
  u(i, 2) = 0.0;
}

bool bad_count(int64_t n) { return n < 0 || n > (int64_t(1) << 31) - 1; }

}  // namespace

extern "C" {

int lpm_farfield_create(lpm_context* ctx, lpm_farfield** out, double theta, int leaf_max,
                        double rho_min) {
  if (!ctx || !out) return fail(LPM_ERR_ARG, "lpm_farfield_create: null argument");
  if (!(theta > 0 && theta < 1)) return fail(LPM_ERR_ARG, "lpm_farfield_create: theta must be in (0, 1)");
  if (leaf_max < 1 || leaf_max > lpm::kMaxLeaf)
    return fail(LPM_ERR_ARG, "lpm_farfield_create: leaf size must be in [1, 64]");
  if (!(rho_min >= 0 && rho_min <= theta))
    return fail(LPM_ERR_ARG, "lpm_farfield_create: rho_min must be in [0, theta]");
  try {
    lpm::DeviceGuard device_guard(ctx->device);
    lpm_farfield* f = new lpm_farfield();
    f->ctx = ctx;
    f->theta = theta;
    f->leaf_max = leaf_max;
    f->rho_min = rho_min;
    *out = f;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_farfield_destroy(lpm_farfield* ff) {
  if (!ff) return LPM_OK;
  try {
    lpm::DeviceGuard device_guard(ff->ctx->device);
    cudaStreamSynchronize(ff->ctx->stream);
    delete ff->net;
    ff->net = nullptr;
    delete ff;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_farfield_set_network(lpm_farfield* ff, int enable) {
  if (!ff) return fail(LPM_ERR_ARG, "null far field");
  if (enable && !ff->trained)
    return fail(LPM_ERR_STATE, "lpm_farfield_set_network: no trained or loaded network");
  ff->use_net = enable != 0;
  return LPM_OK;
}

int lpm_farfield_train(lpm_farfield* ff, int64_t nsamples, int epochs, int batch, double lr,
                       uint64_t seed, int level_min, int level_max, double eps, float* loss) {
  if (!ff) return fail(LPM_ERR_ARG, "null far field");
  if (level_min < 1 || level_max < level_min || level_max > 9)
    return fail(LPM_ERR_ARG, "lpm_farfield_train: levels must satisfy 1 <= min <= max <= 9");
  if (!(lr > 0) || !(eps >= 0)) return fail(LPM_ERR_ARG, "lpm_farfield_train: bad lr or eps");
  if (nsamples < 128 || nsamples > (int64_t(1) << 31) - 1)
    return fail(LPM_ERR_ARG, "lpm_farfield_train: nsamples out of range");
  try {
    lpm::DeviceGuard device_guard(ff->ctx->device);
    lpm::TrainCfg c{nsamples, epochs, batch, lr, seed, level_min, level_max, eps};
    const std::vector<float> h = ff->train(c);
    if (loss)
      for (size_t i = 0; i < h.size(); ++i) loss[i] = h[i];
    ff->use_net = true;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_farfield_get_weights(lpm_farfield* ff, float* w, float* norm) {
  if (!ff || !w || !norm) return fail(LPM_ERR_ARG, "null argument");
  if (ff->w.size() != size_t(lpm::kNParam)) return fail(LPM_ERR_STATE, "no network weights");
  std::copy(ff->w.begin(), ff->w.end(), w);
  std::copy(ff->norm.begin(), ff->norm.end(), norm);
  return LPM_OK;
}

int lpm_farfield_set_weights(lpm_farfield* ff, const float* w, const float* norm) {
  if (!ff || !w || !norm) return fail(LPM_ERR_ARG, "null argument");
  try {
    lpm::DeviceGuard device_guard(ff->ctx->device);
    ff->w.assign(w, w + lpm::kNParam);
    ff->norm.assign(norm, norm + LPM_FF_NNORM);
    ff->upload_net();
    ff->trained = true;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_farfield_grad(lpm_farfield* ff, const float* x, const float* y, int n, float* grad) {
  if (!ff || !x || !y || !grad) return fail(LPM_ERR_ARG, "null argument");
  try {
    lpm::DeviceGuard device_guard(ff->ctx->device);
    ff->grad(x, y, n, grad);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_farfield_velocity(lpm_farfield* ff, lpm_view u, lpm_view x, int64_t nx, lpm_view fx,
                          const double* zeta, const double* area, const uint8_t* mask, int64_t nf,
                          double eps) {
  if (!ff) return fail(LPM_ERR_ARG, "null far field");
  if (bad_count(nx) || bad_count(nf)) return fail(LPM_ERR_ARG, "count out of range [0, 2^31-1]");
  if (nx == 0) return LPM_OK;
  if (!u.p || !x.p || !fx.p || !zeta || !area || !mask) return fail(LPM_ERR_ARG, "null pointer");
  if ((u.stride_i == 0 || x.stride_i == 0) && nx > 1) return fail(LPM_ERR_ARG, "zero row stride");
  if (!(eps >= 0) || !std::isfinite(eps)) return fail(LPM_ERR_ARG, "eps must be finite and >= 0");
  try {
    lpm_context& c = *ff->ctx;
    lpm::DeviceGuard device_guard(c.device);
    c.arena.reset();
    c.arena.reserve(sizeof(int) * (2 * size_t(nf) + 2 * size_t(nf) / 1024 + 8) +
                    sizeof(double4_16a) * size_t(nf + nx) + sizeof(double) * 3 * size_t(nx) + 8192);
    int* slot2src = static_cast<int*>(c.arena.take(sizeof(int) * std::max<int64_t>(nf, 1)));
    int* src2slot = static_cast<int*>(c.arena.take(sizeof(int) * std::max<int64_t>(nf, 1)));
    const int64_t ns = lpm::compact_sources(c, mask, nf, slot2src, src2slot);
    if (ns == 0) {
      k_ff_zero<<<unsigned((nx + 255) / 256), 256, 0, c.stream>>>(nx, lpm::to_view(u));
      c.launches++;
      LPM_CUDA(cudaGetLastError());
      return LPM_OK;
    }
    double4_16a* src = static_cast<double4_16a*>(c.arena.take(sizeof(double4_16a) * ns));
    double4_16a* tgt = static_cast<double4_16a*>(c.arena.take(sizeof(double4_16a) * nx));
    double* w = static_cast<double*>(c.arena.take(sizeof(double) * 3 * nx));
    k_ff_pack_src<<<unsigned((ns + 255) / 256), 256, 0, c.stream>>>(lpm::to_view(fx), zeta, area,
                                                                     src2slot, ns, src);
    k_ff_pack_tgt<<<unsigned((nx + 255) / 256), 256, 0, c.stream>>>(lpm::to_view(x), nx, tgt);
    c.launches += 2;
    std::vector<double4_16a> hs(ns), ht(nx);
    LPM_CUDA(cudaMemcpyAsync(hs.data(), src, sizeof(double4_16a) * ns, cudaMemcpyDeviceToHost, c.stream));
    LPM_CUDA(cudaMemcpyAsync(ht.data(), tgt, sizeof(double4_16a) * nx, cudaMemcpyDeviceToHost, c.stream));
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<double> sx(3 * ns), tx(3 * nx);
    for (int64_t i = 0; i < ns; ++i) sx[3 * i] = hs[i].x, sx[3 * i + 1] = hs[i].y, sx[3 * i + 2] = hs[i].z;
    for (int64_t i = 0; i < nx; ++i) tx[3 * i] = ht[i].x, tx[3 * i + 1] = ht[i].y, tx[3 * i + 2] = ht[i].z;
    ff->build(sx.data(), ns, tx.data(), nx);
    ff->evaluate(tgt, src, w, nx, lpm::chord_c0(3, eps), eps);
    k_ff_velocity<<<unsigned((nx + 255) / 256), 256, 0, c.stream>>>(w, nx, lpm::to_view(x),
                                                                     lpm::to_view(u));
    c.launches++;
    LPM_CUDA(cudaGetLastError());
    lpm::check_device_error(c);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_farfield_stats(lpm_farfield* ff, int64_t* out) {
  if (!ff || !out) return fail(LPM_ERR_ARG, "null argument");
  if (!ff->built()) return fail(LPM_ERR_STATE, "far field: no evaluation yet");
  try {
    lpm::DeviceGuard device_guard(ff->ctx->device);
    ff->counts();
    out[0] = ff->last_far;
    out[1] = ff->last_near;
    out[2] = ff->last_learn;
    out[3] = ff->last_fallback;
    out[4] = ff->d->ncells;
    out[5] = ff->d->nblocks;
    out[6] = ff->last_rows;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_farfield_timing(lpm_farfield* ff, int enable, double* tree_ms, double* net_ms,
                        int64_t* evals) {
  if (!ff) return fail(LPM_ERR_ARG, "null far field");
  try {
    lpm::DeviceGuard device_guard(ff->ctx->device);
    double a = 0, b = 0;
    int64_t n = 0;
    ff->timings(&a, &b, &n);
    if (tree_ms) *tree_ms = a;
    if (net_ms) *net_ms = b;
    if (evals) *evals = n;
    ff->timing = enable != 0;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_octree_stats(const double* src_xyz, int64_t nsrc, const double* tgt_xyz, int64_t ntgt,
                     int leaf_max, int64_t* out) {
  if (!src_xyz || !out || (ntgt > 0 && !tgt_xyz)) return fail(LPM_ERR_ARG, "null argument");
  if (nsrc <= 0 || bad_count(nsrc) || bad_count(ntgt)) return fail(LPM_ERR_ARG, "count out of range");
  try {
    const lpm::TreeTopo t = lpm::build_tree(src_xyz, nsrc, tgt_xyz, ntgt, leaf_max);
    const int64_t nc = int64_t(t.start.size());
    int64_t leaves = 0, max_leaf = 0, in_leaves = 0, bad = 0;
    std::vector<char> seen(size_t(nsrc), 0);
    for (int v : t.perm) {
      if (v < 0 || v >= nsrc || seen[v]) bad++;
      else seen[v] = 1;
    }
    for (int64_t i = 0; i < nc; ++i) {
      if (t.nchild[i] == 0) {
        leaves++;
        in_leaves += t.count[i];
        max_leaf = std::max<int64_t>(max_leaf, t.count[i]);
        continue;
      }
      // children contiguous, covering the parent's range in order
      int64_t pos = t.start[i];
      for (int k = 0; k < t.nchild[i]; ++k) {
        const int ch = t.child0[i] + k;
        if (t.start[ch] != pos || t.count[ch] <= 0 || t.level[ch] != t.level[i] + 1) bad++;
        pos += t.count[ch];
      }
      if (pos != t.start[i] + t.count[i]) bad++;
    }
    int64_t covered = 0, min_fill = lpm::kTargetBlock;
    std::vector<char> tseen(size_t(std::max<int64_t>(ntgt, 1)), 0);
    for (int64_t b = 0; b < t.nblocks; ++b) {
      int64_t fill = 0;
      for (int r = 0; r < lpm::kTargetBlock; ++r) {
        const int v = t.tslot[size_t(b) * lpm::kTargetBlock + r];
        if (v < 0) continue;
        fill++;
        if (v >= ntgt || tseen[v]) bad++;
        else tseen[v] = 1;
      }
      covered += fill;
      min_fill = std::min(min_fill, fill);
    }
    out[0] = nc;
    out[1] = leaves;
    out[2] = max_leaf;
    out[3] = t.max_level;
    out[4] = t.nblocks;
    out[5] = t.nblocks ? min_fill : 0;
    out[6] = covered;
    out[7] = in_leaves;
    out[8] = bad;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_mesh_build_device(lpm_context* ctx, int kind, int level, double radius, double* vx,
                          double* fx, double* farea, uint8_t* fmask) {
  if (!ctx || !vx || !fx || !farea || !fmask) return fail(LPM_ERR_ARG, "null argument");
  if (kind < LPM_MESH_ICOS_TRI || kind > LPM_MESH_QUAD_RECT) return fail(LPM_ERR_ARG, "unknown mesh kind");
  if (level < 0 || level > 10) return fail(LPM_ERR_ARG, "mesh level out of range [0, 10]");
  if (!(radius > 0) || !std::isfinite(radius)) return fail(LPM_ERR_ARG, "radius must be positive");
  try {
    lpm::DeviceGuard device_guard(ctx->device);
    lpm::mesh_build_device(*ctx, kind, level, radius, vx, fx, farea, fmask);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_tc_selftest(lpm_context* ctx, const float* A, const float* B, float* D, int N, int K,
                    int a_mn, int b_mn) {
  if (!ctx || !A || !B || !D) return fail(LPM_ERR_ARG, "null argument");
  try {
    lpm::DeviceGuard device_guard(ctx->device);
    lpm::tc_selftest(*ctx, A, B, D, N, K, a_mn, b_mn);
    lpm::check_device_error(*ctx);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

}  // extern "C"

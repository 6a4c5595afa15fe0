// mesh_dev.cu -- uniform mesh refinement on the device.
//
// Produces the same arrays as the host generator (mesh.cpp): the seed's
// faces are divided level by level in index order, four children appended
// per divided face, the divided face keeping its slot with mask 1 and area 0
// (src/mesh/lpm_polymesh2d_impl.hpp:26-42, src/mesh/lpm_faces_impl.hpp
// :285-575).  The serial rule "an edge's midpoint becomes a new vertex the
// first time the edge is divided" (src/mesh/lpm_edges.cpp:59-96) fixes the
// vertex numbering; per level it is evaluated in parallel:
//   1. every (leaf face j, local edge e) inserts its edge into a hash table
//      and atomicMin's the code 4j + e into the edge's owner slot;
//   2. face j counts the edges it owns (+1 for a quad's centre vertex);
//   3. an exclusive scan of the counts gives each face its first new vertex,
//      so the numbering is the serial first-encounter order;
//   4. owners write their midpoint vertices (and quads their centre);
//   5. every face looks up its midpoints and writes its four children
//      (barycentre and area as in mesh.cpp) at slot stop + 4 j + k.
// FP64 arithmetic uses non-contracting intrinsics in the host's operation
// order, so positions are bitwise equal to a host build compiled without
// contraction; areas go through tan/atan, whose last bits may differ.
#include <cmath>
#include <vector>

#include <cuda_runtime.h>

#include "lpm_host.hpp"

namespace lpm {
namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

struct Geo {
  int ndim;
  bool sphere;
};

__device__ void normalize3(double* p) {
  const double r = __dsqrt_rn(da(da(dm(p[0], p[0]), dm(p[1], p[1])), dm(p[2], p[2])));
  const double s = __ddiv_rn(1.0, r);
  p[0] = dm(p[0], s);
  p[1] = dm(p[1], s);
  p[2] = dm(p[2], s);
}

__device__ double sdistance(const double* a, const double* b) {
  const double cp0 = ds(dm(a[1], b[2]), dm(a[2], b[1]));
  const double cp1 = ds(dm(a[2], b[0]), dm(a[0], b[2]));
  const double cp2 = ds(dm(a[0], b[1]), dm(a[1], b[0]));
  const double dp = da(da(dm(a[0], b[0]), dm(a[1], b[1])), dm(a[2], b[2]));
  return atan2(__dsqrt_rn(da(da(dm(cp0, cp0), dm(cp1, cp1)), dm(cp2, cp2))), dp);
}

__device__ double tri_area(const Geo& g, const double* a, const double* b, const double* c) {
  if (!g.sphere) {
    const double ar = ds(dm(ds(b[0], a[0]), ds(c[1], a[1])), dm(ds(b[1], a[1]), ds(c[0], a[0])));
    return dm(0.5, fabs(ar));
  }
  const double s1 = sdistance(a, b), s2 = sdistance(b, c), s3 = sdistance(c, a);
  const double hp = dm(0.5, da(da(s1, s2), s3));
  double zz = dm(dm(dm(tan(dm(0.5, hp)), tan(dm(0.5, ds(hp, s1)))), tan(dm(0.5, ds(hp, s2)))),
                 tan(dm(0.5, ds(hp, s3))));
  if (fabs(zz) < 2.220446049250313e-16) zz = 0;
  return dm(4.0, atan(__dsqrt_rn(zz)));
}

// Barycentre (normalised on the sphere) and polygon area of a face.
__device__ void face_geometry(const Geo& g, const double* vx, const int* vs, int n, double* c,
                              double* area) {
  c[0] = c[1] = c[2] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < g.ndim; ++k) c[k] = da(c[k], vx[int64_t(g.ndim) * vs[i] + k]);
  const double s = __ddiv_rn(1.0, double(n));
  for (int k = 0; k < g.ndim; ++k) c[k] = dm(c[k], s);
  if (g.sphere) normalize3(c);
  double ar = 0.0;
  for (int i = 0; i < n; ++i)
    ar = da(ar, tri_area(g, c, vx + int64_t(g.ndim) * vs[i], vx + int64_t(g.ndim) * vs[(i + 1) % n]));
  *area = ar;
}

constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ unsigned long long edge_key(int a, int b) {
  const unsigned lo = unsigned(a < b ? a : b), hi = unsigned(a < b ? b : a);
  return (static_cast<unsigned long long>(hi) << 32) | lo;
}
__device__ __forceinline__ unsigned slot_of(unsigned long long key, unsigned mask) {
  return unsigned((key * 0x9E3779B97F4A7C15ull) >> 32) & mask;
}

// 1. insert the edges of every leaf face, owner = min(4 j + e)
__global__ void k_mesh_edges(const int* __restrict__ fv, int nl, int nfv,
                             unsigned long long* __restrict__ keys, int* __restrict__ owner,
                             unsigned mask, int* __restrict__ err) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= int64_t(nl) * nfv) return;
  const int j = int(i / nfv), e = int(i % nfv);
  const unsigned long long key = edge_key(fv[j * nfv + e], fv[j * nfv + (e + 1) % nfv]);
  unsigned s = slot_of(key, mask);
  for (unsigned probe = 0; probe <= mask; ++probe) {
    const unsigned long long prev = atomicCAS(&keys[s], kEmpty, key);
    if (prev == kEmpty || prev == key) {
      atomicMin(&owner[s], 4 * j + e);
      return;
    }
    s = (s + 1) & mask;
  }
  atomicExch(err, 1);  // table full (capacity is twice the references: unreachable)
}

__device__ __forceinline__ int find_slot(const unsigned long long* keys, unsigned long long key,
                                         unsigned mask) {
  unsigned s = slot_of(key, mask);
  for (unsigned probe = 0; probe <= mask; ++probe) {
    const unsigned long long k = keys[s];
    if (k == key) return int(s);
    if (k == kEmpty) return -1;
    s = (s + 1) & mask;
  }
  return -1;
}

// 2. new vertices per face: owned edges (+ a quad's centre)
__global__ void k_mesh_count(const int* __restrict__ fv, int nl, int nfv,
                             const unsigned long long* __restrict__ keys,
                             const int* __restrict__ owner, unsigned mask, int* __restrict__ cnt) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nl) return;
  int c = nfv == 4 ? 1 : 0;
  for (int e = 0; e < nfv; ++e) {
    const int s = find_slot(keys, edge_key(fv[j * nfv + e], fv[j * nfv + (e + 1) % nfv]), mask);
    if (s >= 0 && owner[s] == 4 * j + e) ++c;
  }
  cnt[j] = c;
}

// 3. exclusive scan (three passes: per-block sums, scan of the block sums in
// one CTA, add)
constexpr int kScanBlock = 1024;
__global__ void k_scan_local(int* __restrict__ v, int n, int* __restrict__ bsum) {
  __shared__ int sh[kScanBlock];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int x = i < n ? v[i] : 0;
  sh[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) v[i] = sh[threadIdx.x] - x;  // exclusive within the block
  if (threadIdx.x == kScanBlock - 1) bsum[blockIdx.x] = sh[threadIdx.x];
}
__global__ void k_scan_blocks(int* __restrict__ bsum, int nb, int* __restrict__ total) {
  if (threadIdx.x != 0) return;
  int run = 0;
  for (int b = 0; b < nb; ++b) {
    const int x = bsum[b];
    bsum[b] = run;
    run += x;
  }
  *total = run;
}
__global__ void k_scan_add(int* __restrict__ v, int n, const int* __restrict__ bsum) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) v[i] += bsum[blockIdx.x];
}

// 4. owners create the midpoint vertices; quads their centre
__global__ void k_mesh_vertices(Geo g, const int* __restrict__ fv, int nl, int nfv, int64_t start,
                                const unsigned long long* __restrict__ keys,
                                const int* __restrict__ owner, unsigned mask,
                                const int* __restrict__ base, int nv0, double* __restrict__ vx,
                                const double* __restrict__ fx, int* __restrict__ vid) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nl) return;
  int next = nv0 + base[j];
  for (int e = 0; e < nfv; ++e) {
    const int a = fv[j * nfv + e], b = fv[j * nfv + (e + 1) % nfv];
    const int s = find_slot(keys, edge_key(a, b), mask);
    if (s < 0 || owner[s] != 4 * j + e) continue;
    double m[3] = {0, 0, 0};
    for (int k = 0; k < g.ndim; ++k)
      m[k] = dm(0.5, da(vx[int64_t(g.ndim) * a + k], vx[int64_t(g.ndim) * b + k]));
    if (g.sphere) normalize3(m);
    for (int k = 0; k < g.ndim; ++k) vx[int64_t(g.ndim) * next + k] = m[k];
    vid[s] = next;
    ++next;
  }
  if (nfv == 4)
    for (int k = 0; k < g.ndim; ++k) vx[int64_t(g.ndim) * next + k] = fx[g.ndim * (start + j) + k];
}

// 5. children of every leaf face
__global__ void k_mesh_children(Geo g, const int* __restrict__ fv, int nl, int nfv, int64_t start,
                                int64_t stop, const unsigned long long* __restrict__ keys,
                                unsigned mask, const int* __restrict__ vid,
                                const int* __restrict__ base, const int* __restrict__ cnt,
                                int nv0, const double* __restrict__ vx, double* __restrict__ fx,
                                double* __restrict__ farea, uint8_t* __restrict__ fmask,
                                int* __restrict__ fv_next, int* __restrict__ err) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nl) return;
  int p[4], m[4];
  for (int e = 0; e < nfv; ++e) p[e] = fv[j * nfv + e];
  for (int e = 0; e < nfv; ++e) {
    const int s = find_slot(keys, edge_key(p[e], p[(e + 1) % nfv]), mask);
    if (s < 0) {
      atomicExch(err, 1);
      return;
    }
    m[e] = vid[s];
  }
  int kids[4][4];
  if (nfv == 3) {
    const int k0[3] = {p[0], m[0], m[2]}, k1[3] = {m[0], p[1], m[1]};
    const int k2[3] = {m[2], m[1], p[2]}, k3[3] = {m[1], m[2], m[0]};
    for (int i = 0; i < 3; ++i) {
      kids[0][i] = k0[i];
      kids[1][i] = k1[i];
      kids[2][i] = k2[i];
      kids[3][i] = k3[i];
    }
  } else {
    const int ci = nv0 + base[j] + cnt[j] - 1;  // the centre comes after the owned midpoints
    for (int i = 0; i < 4; ++i) {
      kids[i][i] = p[i];
      kids[i][(i + 1) % 4] = m[i];
      kids[i][(i + 2) % 4] = ci;
      kids[i][(i + 3) % 4] = m[(i + 3) % 4];
    }
  }
  for (int k = 0; k < 4; ++k) {
    const int64_t f = stop + 4 * int64_t(j) + k;
    double c[3], ar;
    face_geometry(g, vx, kids[k], nfv, c, &ar);
    for (int d = 0; d < g.ndim; ++d) fx[g.ndim * f + d] = c[d];
    farea[f] = ar;
    fmask[f] = 0;
    for (int i = 0; i < nfv; ++i) fv_next[(4 * j + k) * nfv + i] = kids[k][i];
  }
  farea[start + j] = 0.0;
  fmask[start + j] = 1;
}

__global__ void k_fill_u64(unsigned long long* p, int64_t n, unsigned long long v) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) p[i] = v;
}
__global__ void k_fill_i32(int* p, int64_t n, int v) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) p[i] = v;
}

}  // namespace

// vx, fx, farea, fmask: device arrays sized by mesh_sizes (AoS, ndim per row).
void mesh_build_device(lpm_context& ctx, int kind, int level, double radius, double* vx,
                       double* fx, double* farea, uint8_t* fmask) {
  int64_t nv_all, nf_all;
  mesh_sizes(kind, level, &nv_all, &nf_all);
  MeshSeed seed;
  mesh_seed(kind, radius, seed);
  const Geo g{seed.ndim, seed.sphere};
  const int nfv = seed.nfv;
  const int64_t nf0 = int64_t(seed.area.size());
  const int64_t nv_seed = int64_t(seed.vx.size()) / g.ndim;
  cudaStream_t st = ctx.stream;
  // scratch: face vertex lists of two levels, hash table, counts
  const int64_t nl_max = nf0 << (2 * std::max(level - 1, 0));  // leaves divided last
  size_t cap = 1;
  while (cap < size_t(2 * nl_max * nfv)) cap <<= 1;
  const size_t fvbytes = sizeof(int) * size_t(nl_max) * nfv * 4 + 64;  // one level's children
  const size_t need = 2 * fvbytes + (sizeof(unsigned long long) + 2 * sizeof(int)) * cap +
                      2 * (sizeof(int) * size_t(nl_max) + 64) +
                      sizeof(int) * (size_t(nl_max) / kScanBlock + 8) + 8 * 256;
  ctx.arena.reset();
  ctx.arena.reserve(need);
  int* fva = static_cast<int*>(ctx.arena.take(fvbytes));
  int* fvb = static_cast<int*>(ctx.arena.take(fvbytes));
  auto* keys = static_cast<unsigned long long*>(ctx.arena.take(sizeof(unsigned long long) * cap));
  int* owner = static_cast<int*>(ctx.arena.take(sizeof(int) * cap));
  int* vid = static_cast<int*>(ctx.arena.take(sizeof(int) * cap));
  int* cnt = static_cast<int*>(ctx.arena.take(sizeof(int) * size_t(nl_max) + 64));
  int* base = static_cast<int*>(ctx.arena.take(sizeof(int) * size_t(nl_max) + 64));
  int* bsum = static_cast<int*>(ctx.arena.take(sizeof(int) * (size_t(nl_max) / kScanBlock + 8)));
  int* total = bsum + (nl_max / kScanBlock + 4);
  LPM_CUDA(cudaMemcpyAsync(vx, seed.vx.data(), sizeof(double) * seed.vx.size(), cudaMemcpyHostToDevice, st));
  LPM_CUDA(cudaMemcpyAsync(fx, seed.fx.data(), sizeof(double) * seed.fx.size(), cudaMemcpyHostToDevice, st));
  LPM_CUDA(cudaMemcpyAsync(farea, seed.area.data(), sizeof(double) * nf0, cudaMemcpyHostToDevice, st));
  LPM_CUDA(cudaMemsetAsync(fmask, 0, nf0, st));
  LPM_CUDA(cudaMemcpyAsync(fva, seed.fverts.data(), sizeof(int) * seed.fverts.size(), cudaMemcpyHostToDevice, st));
  int64_t start = 0, stop = nf0, nv = nv_seed;
  for (int l = 0; l < level; ++l) {
    const int nl = int(stop - start);
    size_t c = 1;
    while (c < size_t(2 * int64_t(nl) * nfv)) c <<= 1;
    const unsigned mask = unsigned(c - 1);
    k_fill_u64<<<unsigned((c + 255) / 256), 256, 0, st>>>(keys, int64_t(c), kEmpty);
    k_fill_i32<<<unsigned((c + 255) / 256), 256, 0, st>>>(owner, int64_t(c), 0x7fffffff);
    const int64_t refs = int64_t(nl) * nfv;
    k_mesh_edges<<<unsigned((refs + 255) / 256), 256, 0, st>>>(fva, nl, nfv, keys, owner, mask, ctx.d_err);
    k_mesh_count<<<(nl + 255) / 256, 256, 0, st>>>(fva, nl, nfv, keys, owner, mask, cnt);
    LPM_CUDA(cudaMemcpyAsync(base, cnt, sizeof(int) * nl, cudaMemcpyDeviceToDevice, st));
    const int nb = (nl + kScanBlock - 1) / kScanBlock;
    k_scan_local<<<nb, kScanBlock, 0, st>>>(base, nl, bsum);
    k_scan_blocks<<<1, 32, 0, st>>>(bsum, nb, total);
    k_scan_add<<<nb, kScanBlock, 0, st>>>(base, nl, bsum);
    k_mesh_vertices<<<(nl + 255) / 256, 256, 0, st>>>(g, fva, nl, nfv, start, keys, owner, mask,
                                                      base, int(nv), vx, fx, vid);
    k_mesh_children<<<(nl + 255) / 256, 256, 0, st>>>(g, fva, nl, nfv, start, stop, keys, mask,
                                                      vid, base, cnt, int(nv), vx, fx, farea,
                                                      fmask, fvb, ctx.d_err);
    ctx.launches += 9;
    int h_total = 0;
    LPM_CUDA(cudaMemcpyAsync(&h_total, total, sizeof(int), cudaMemcpyDeviceToHost, st));
    LPM_CUDA(cudaStreamSynchronize(st));
    nv += h_total;
    start = stop;
    stop = stop + 4 * int64_t(nl);
    std::swap(fva, fvb);
  }
  LPM_CUDA(cudaGetLastError());
  check_device_error(ctx);
  if (nv != nv_all || stop != nf_all)
    throw Error(LPM_ERR_STATE, "device mesh: vertex or face count differs from the tree formula");
}

}  // namespace lpm

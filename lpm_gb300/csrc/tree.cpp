// tree.cpp -- host construction of the source octree and the target blocks.
//
// Points are ordered along a Morton (Z-order) curve of a cube that bounds
// them, 21 bits per axis.  Cells are the nodes of the implied octree: a cell
// with more than leaf_max points is split by the next three key bits into
// its non-empty octants.  Cells are numbered breadth first, so the children
// of a cell are contiguous; each cell is a contiguous range of the sorted
// order.  Targets are Morton-sorted the same way and cut into target blocks
// of at most kTargetBlock targets (padded to kTargetBlock rows): the leaves of
// a target octree, consecutive small sibling leaves packed into one block, so
// no block straddles a jump of the curve and blocks stay well filled.
//
// The reference has no working octree (its LpmOctree/LpmNodeArray sources are
// not built and lpm_cpu_tree indexes points by loop index); this is the
// project's own structure for the far-field evaluation.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <system_error>
#include <thread>
#include <vector>

#include "farfield.hpp"

namespace lpm {

namespace {

uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffffULL;
  v = (v | (v << 32)) & 0x1f00000000ffffULL;
  v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
  v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}

struct Box {
  double lo[3], scale;
};

Box bounding_cube(const double* a, int64_t n, const double* b, int64_t m) {
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  auto take = [&](const double* p, int64_t k) {
    for (int64_t i = 0; i < k; ++i)
      for (int c = 0; c < 3; ++c) {
        lo[c] = std::min(lo[c], p[3 * i + c]);
        hi[c] = std::max(hi[c], p[3 * i + c]);
      }
  };
  take(a, n);
  take(b, m);
  double ext = 0;
  for (int c = 0; c < 3; ++c) ext = std::max(ext, hi[c] - lo[c]);
  ext = ext * (1 + 1e-9) + 1e-12;
  Box bx;
  for (int c = 0; c < 3; ++c) bx.lo[c] = lo[c] - 1e-12;
  bx.scale = double(1 << 21) / ext;
  return bx;
}

uint64_t key_of(const Box& bx, const double* p) {
  uint64_t k = 0;
  for (int c = 0; c < 3; ++c) {
    double q = (p[c] - bx.lo[c]) * bx.scale;
    uint64_t iq = q <= 0 ? 0 : std::min<uint64_t>(uint64_t(q), (1u << 21) - 1);
    k |= spread3(iq) << (2 - c);
  }
  return k;
}

// Runs jobs(0..count-1) on their own threads; a job whose thread cannot be
// created (std::system_error, e.g. under a container's thread limit) runs on
// the calling thread instead.  Returns after every job has finished.
template <class Job>
void run_jobs(int count, const Job& job) {
  std::vector<std::thread> th;
  th.reserve(count);
  for (int i = 0; i < count; ++i) {
    try {
      th.emplace_back(job, i);
    } catch (const std::system_error&) {
      job(i);
    }
  }
  for (auto& t : th) t.join();
}

// Sorts (key, index) pairs on up to 16 host threads: equal chunks sorted
// concurrently, then merged pairwise.  The pairs are totally ordered (ties
// in key broken by index), so the result is the single-threaded one.
void parallel_sort(std::vector<std::pair<uint64_t, int>>& v) {
  const int64_t n = int64_t(v.size());
  const int hw = int(std::min(16u, std::max(1u, std::thread::hardware_concurrency())));
  if (n < (int64_t(1) << 16) || hw == 1) {
    std::sort(v.begin(), v.end());
    return;
  }
  int p = 1;
  while (p * 2 <= hw) p *= 2;
  std::vector<int64_t> cut(p + 1);
  for (int i = 0; i <= p; ++i) cut[i] = n * i / p;
  run_jobs(p, [&v, &cut](int i) { std::sort(v.begin() + cut[i], v.begin() + cut[i + 1]); });
  for (int w = 1; w < p; w *= 2) {
    const int merges = (p - w + 2 * w - 1) / (2 * w);  // i = 0, 2w, ... with i + w < p
    run_jobs(merges, [&v, &cut, w, p](int m) {
      const int i = 2 * w * m;
      std::inplace_merge(v.begin() + cut[i], v.begin() + cut[i + w],
                         v.begin() + cut[std::min(i + 2 * w, p)]);
    });
  }
}

std::vector<int> sorted_order(const Box& bx, const double* p, int64_t n, std::vector<uint64_t>& keys) {
  std::vector<std::pair<uint64_t, int>> kv(n);
  for (int64_t i = 0; i < n; ++i) kv[i] = {key_of(bx, p + 3 * i), int(i)};
  parallel_sort(kv);
  std::vector<int> perm(n);
  keys.resize(n);
  for (int64_t i = 0; i < n; ++i) {
    perm[i] = kv[i].second;
    keys[i] = kv[i].first;
  }
  return perm;
}

}  // namespace

TreeTopo build_tree(const double* src_xyz, int64_t nsrc, const double* tgt_xyz, int64_t ntgt,
                    int leaf_max) {
  if (nsrc <= 0) throw Error(LPM_ERR_ARG, "build_tree: no sources");
  if (leaf_max < 1 || leaf_max > kMaxLeaf) throw Error(LPM_ERR_ARG, "build_tree: leaf size out of range");
  TreeTopo t;
  const Box bx = bounding_cube(src_xyz, nsrc, tgt_xyz, ntgt);
  std::vector<uint64_t> keys;
  t.perm = sorted_order(bx, src_xyz, nsrc, keys);
  // breadth-first split
  struct C {
    int start, count, level;
  };
  std::vector<C> cells{{0, int(nsrc), 0}};
  t.child0.push_back(-1);
  t.nchild.push_back(0);
  for (size_t i = 0; i < cells.size(); ++i) {
    const C c = cells[i];
    if (c.count <= leaf_max || c.level >= 21) continue;
    const int shift = 3 * (20 - c.level);
    int b = c.start;
    const int e = c.start + c.count;
    t.child0[i] = int(cells.size());
    int nch = 0;
    while (b < e) {
      const uint64_t oct = (keys[b] >> shift) & 7;
      int j = b;
      while (j < e && ((keys[j] >> shift) & 7) == oct) ++j;
      cells.push_back({b, j - b, c.level + 1});
      t.child0.push_back(-1);
      t.nchild.push_back(0);
      ++nch;
      b = j;
    }
    t.nchild[i] = nch;
  }
  const size_t nc = cells.size();
  t.start.resize(nc);
  t.count.resize(nc);
  t.level.resize(nc);
  for (size_t i = 0; i < nc; ++i) {
    t.start[i] = cells[i].start;
    t.count[i] = cells[i].count;
    t.level[i] = cells[i].level;
    if (t.nchild[i] == 0) t.child0[i] = -1;
    t.max_level = std::max(t.max_level, cells[i].level);
  }
  // targets: Morton order cut into the leaves of an octree with at most
  // kTargetBlock targets each, so that no block straddles a jump of the curve
  std::vector<uint64_t> tkeys;
  std::vector<int> tperm = ntgt > 0 ? sorted_order(bx, tgt_xyz, ntgt, tkeys) : std::vector<int>{};
  std::vector<std::pair<int, int>> blocks;
  std::vector<C> work;
  if (ntgt > 0) work.push_back({0, int(ntgt), 0});
  while (!work.empty()) {
    const C c = work.back();
    work.pop_back();
    if (c.count <= kTargetBlock || c.level >= 21) {  // a leaf, or packed siblings
      for (int b = 0; b < c.count; b += kTargetBlock)
        blocks.push_back({c.start + b, std::min(kTargetBlock, c.count - b)});
      continue;
    }
    const int shift = 3 * (20 - c.level);
    std::vector<C> kids;
    int b = c.start;
    const int e = c.start + c.count;
    while (b < e) {
      const uint64_t oct = (tkeys[b] >> shift) & 7;
      int j = b;
      while (j < e && ((tkeys[j] >> shift) & 7) == oct) ++j;
      kids.push_back({b, j - b, c.level + 1});
      b = j;
    }
    // consecutive small siblings share a block (they lie in the same parent
    // octant); larger ones are split further
    std::vector<C> split;
    for (size_t k = 0; k < kids.size();) {
      if (kids[k].count > kTargetBlock) {
        split.push_back(kids[k++]);
        continue;
      }
      int s0 = kids[k].start, n0 = 0;
      while (k < kids.size() && kids[k].count <= kTargetBlock && n0 + kids[k].count <= kTargetBlock)
        n0 += kids[k++].count;
      split.push_back({s0, n0, 99});  // level 99: emit as one block
    }
    for (auto it = split.rbegin(); it != split.rend(); ++it) work.push_back(*it);
  }
  t.nblocks = int64_t(blocks.size());
  t.tslot.assign(size_t(t.nblocks) * kTargetBlock, -1);
  for (size_t k = 0; k < blocks.size(); ++k)
    for (int r = 0; r < blocks[k].second; ++r)
      t.tslot[k * kTargetBlock + r] = tperm[blocks[k].first + r];
  t.ntgt = ntgt;
  t.nsrc = nsrc;
  return t;
}

}  // namespace lpm

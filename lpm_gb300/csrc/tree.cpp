// tree.cpp -- host construction of the source octree and the target blocks.
//
// Points are ordered along a Morton (Z-order) curve of a cube that bounds
// them, 21 bits per axis.  Cells are the nodes of the implied octree: a cell
// with more than leaf_max points is split by the next three key bits into
// its non-empty octants.  Cells are numbered breadth first, so the children
// of a cell are contiguous; each cell is a contiguous range of the sorted
// order.  Targets are Morton-sorted the same way and cut into target blocks
// of 96 to kTargetBlock consecutive targets (padded to kTargetBlock rows),
// each cut at the coarsest octree boundary of its window.
//
// The reference has no working octree (its LpmOctree/LpmNodeArray sources are
// not built and lpm_cpu_tree indexes points by loop index); this is the
// project's own structure for the far-field evaluation.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <stdexcept>
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

std::vector<int> sorted_order(const Box& bx, const double* p, int64_t n, std::vector<uint64_t>& keys) {
  std::vector<std::pair<uint64_t, int>> kv(n);
  for (int64_t i = 0; i < n; ++i) kv[i] = {key_of(bx, p + 3 * i), int(i)};
  std::sort(kv.begin(), kv.end());
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
  // targets: Morton order cut into blocks of 96..kTargetBlock consecutive
  // targets, each cut placed at the coarsest octree boundary in the window
  // (the largest key difference), so blocks stay full and do not straddle a
  // large jump of the curve
  std::vector<uint64_t> tkeys;
  std::vector<int> tperm = ntgt > 0 ? sorted_order(bx, tgt_xyz, ntgt, tkeys) : std::vector<int>{};
  std::vector<std::pair<int, int>> blocks;
  for (int64_t b0 = 0; b0 < ntgt;) {
    int64_t cut = std::min<int64_t>(ntgt, b0 + kTargetBlock);
    if (cut < ntgt) {
      int best = 65;
      for (int64_t p = b0 + kTargetBlock * 3 / 4; p <= b0 + kTargetBlock; ++p) {
        const uint64_t x = tkeys[p - 1] ^ tkeys[p];
        const int lz = x ? __builtin_clzll(x) : 64;
        if (lz <= best) {  // coarser (or equal, later) boundary
          best = lz;
          cut = p;
        }
      }
    }
    blocks.push_back({int(b0), int(cut - b0)});
    b0 = cut;
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

// farfield.hpp -- octree far field for the BVE sphere velocity with a learned
// correction (host side).  Device code: farfield.cu (tree evaluation),
// mlp.cu (tcgen05 network, training, training samples).
#pragma once

#include <cstdint>
#include <vector>

#include "lpm_host.hpp"

namespace lpm {

constexpr int kMaxLeaf = 64;        // largest leaf the kernels stage
constexpr int kTargetBlock = 128;   // targets per block = rows of one MMA tile
// List capacities per target block (28 KB of lists per 128 targets).  A block
// whose lists overflow is summed directly; at icosahedral level 8 these hold
// every block's lists down to theta = 0.2 (with 640 near leaves, 2 blocks
// overflowed at theta = 0.26 and 30 at 0.2, and their direct sums doubled the
// evaluation time).
constexpr int kFarCap = 2048;       // far cells per target block
constexpr int kNearCap = 4096;      // near leaves per target block
constexpr int kLearnCap = 1024;     // learned (cell, block) pairs per block
constexpr int kExactMax = 32;       // accepted cells with fewer points are summed exactly

// Cell record: kCellF floats per cell.
//  [0..2] centre c (mean of the points), [3] |c|, [4] radius h (max |y - c|),
//  [5] S = sum |g|, [6] sum g, [7] count,
//  [8..16] frame rows e1, e2, n (n = c/|c|),
//  [17..51] moments M_b = sum g d^b about c in the cell frame, b over the
//           35 monomials of degree <= 4 (degree, then exponents descending),
//  [52..61] traced moments sum g d^b |d|^2 for |b| <= 2, [62] sum g |d|^4,
//  [64..98] complex moments sum g z^p conj(z)^q w^k (z = d1 + i d2, w = d3),
//           p >= q, p+q+k <= 4, normalised by S h^(p+q+k): 35 reals.
constexpr int kCellF = 112;
constexpr int kCellM = 17, kCellN1 = 52, kCellN2 = 62, kCellC = 64;

// Network: 48 inputs -> 128 -> 128 -> 128 -> 16 (3 used), SiLU, BF16
// weights and activations, FP32 accumulation.  Input 40 and hidden unit 127
// of every layer are the constant 1, so the column of the next weight matrix
// that multiplies them is that layer's bias.
constexpr int kIn = 48, kHid = 128, kOut = 16;
constexpr int kBiasIn = 40, kBiasHid = 127;
constexpr int kW1 = kHid * kIn, kW2 = kHid * kHid, kW3 = kHid * kHid, kW4 = kOut * kHid;
constexpr int kNParam = kW1 + kW2 + kW3 + kW4;  // 40960 FP32 master weights
constexpr int kNFeat = 41;                      // features before padding (incl. bias)

struct TreeTopo {
  int64_t nsrc = 0, ntgt = 0;
  std::vector<int> perm;   // sorted source position -> source index
  int64_t nblocks = 0;     // target blocks (leaves of the target octree)
  std::vector<int> tslot;  // block * 128 + row -> target index, or -1 (padding)
  std::vector<int> start, count, child0, nchild, level;
  int max_level = 0;
};

TreeTopo build_tree(const double* src_xyz, int64_t nsrc, const double* tgt_xyz, int64_t ntgt,
                    int leaf_max);

struct FFDevice;  // tree buffers (farfield_dev.cuh)
struct FFNet;     // network buffers (farfield_dev.cuh)

struct TrainCfg {
  int64_t nsamples;
  int epochs;
  int batch;
  double lr;
  uint64_t seed;
  int level_min, level_max;
  double eps;
};

}  // namespace lpm

struct lpm_farfield {
  lpm_context* ctx = nullptr;
  double theta = 0.5, rho_min = 0.25;
  int leaf_max = 64;
  bool use_net = false;
  bool trained = false;
  lpm::FFDevice* d = nullptr;
  lpm::FFNet* net = nullptr;
  // network (host copy of the FP32 master weights and input normalisation)
  std::vector<float> w;       // kNParam
  std::vector<float> norm;    // mu[48], isd[48], out_scale
  int64_t last_far = 0, last_near = 0, last_learn = 0, last_fallback = 0, last_rows = 0;
  // optional CUDA-event timing of evaluations (not inside graph capture)
  bool timing = false;
  std::vector<void*> events;  // cudaEvent_t triples: start, tree done, network done
  void timings(double* tree_ms, double* net_ms, int64_t* evals);

  ~lpm_farfield();
  // Tree over the sources (nsrc x 3, host) and targets (ntgt x 3, host).
  void build(const double* src_xyz, int64_t nsrc, const double* tgt_xyz, int64_t ntgt);
  bool built() const;
  // w[c * wstride + t] = sum over sources of g (x_t - y) / (|x_t - y|^2 + c0)
  // up to terms parallel to x_t (the chord-form sum whose cross product with
  // x_t gives the velocity), for packed double4_16a targets (x, y, z, _) and
  // sources (x, y, z, g) in the order given to build().
  void evaluate(const void* tgt, const void* src, double* wout, int64_t wstride, double c0,
                double eps);
  void upload_net();
  void init_net(uint64_t seed);
  std::vector<float> train(const lpm::TrainCfg& cfg);
  // one tile's parameter gradients (grad check)
  void grad(const float* x_host, const float* y_host, int n, float* g_host);
  void counts();
};

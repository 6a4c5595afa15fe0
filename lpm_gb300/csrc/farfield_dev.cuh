// farfield_dev.cuh -- device buffers of the octree far field and the launch
// entry points shared by farfield.cu and mlp.cu.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "farfield.hpp"

namespace lpm {

// Tree topology and per-evaluation buffers (one tree).
struct FFDevice {
  int64_t nsrc = 0, ntgt = 0, nblocks = 0;
  int ncells = 0;
  float rmax = 1e30f;  // bound on |target| (with margin) at the last tree build
  int* perm = nullptr;    // sorted source -> packed source index
  int* tslot = nullptr;   // block * 128 + row -> packed target index or -1
  int4* cells = nullptr;  // (start, count, first child, child count)
  float4* ys = nullptr;   // sorted sources (x, y, z, g), FP32
  float* cd = nullptr;    // cell records, kCellF floats each
  float4* xt = nullptr;   // sorted targets (x, y, z, valid), nblocks * 128
  float4* box = nullptr;  // target block centre and radius
  int *far = nullptr, *near = nullptr, *lrn = nullptr;  // per-block lists
  int4* cnt = nullptr;    // (far, near, learned, overflow) per block
  int* counter = nullptr; // [0] work counter of the network kernel, [2..3] rows (u64)
  std::vector<void*> allocs;
  ~FFDevice();
  void* alloc(size_t bytes);
};

// Network weights on the device: BF16 in the tensor-core tile layout
// (W1 128x48, W2 128x128, W3 128x128, W4 16x128, each row-major in core
// matrices) and the input normalisation (mu[48], isd[48], output scale).
struct FFNet {
  uint16_t* wbf = nullptr;
  float* norm = nullptr;
  std::vector<void*> allocs;
  ~FFNet();
  void* alloc(size_t bytes);
};

void ff_launch_tree(lpm_context& ctx, FFDevice& d, const void* tgt, const void* src, double* wout,
                    int64_t wstride, double c0, double theta, double rho_min, bool learn);
// Shared-memory limits of the network kernels (call outside stream capture,
// on the current device).
void ff_prepare_kernels();
// Cell records of a sorted source array (one CTA per cell).
void ff_cells(lpm_context& ctx, const float4* ys, const int4* cells, int ncells, float* cd);
// tcgen05 operand-layout self-test (device pointers, see mlp.cu).
void tc_selftest(lpm_context& ctx, const float* A, const float* B, float* D, int N, int K, int amn,
                 int bmn);
void ff_launch_mlp(lpm_context& ctx, FFDevice& d, FFNet& net, const float* norm, double* wout,
                   int64_t wstride, double eps, double rho_min);

}  // namespace lpm

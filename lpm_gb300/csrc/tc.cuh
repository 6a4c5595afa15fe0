// tc.cuh -- fifth-generation tensor core (tcgen05) building blocks for sm_103a.
//
// Operands live in shared memory without swizzle, in the canonical
// "core matrix" layout: a core matrix is 8 rows x 16 bytes (8 bf16), stored
// as 128 contiguous bytes.  A tile of R rows x C bf16 columns is stored as
// (R/8) x (C/8) core matrices, column-group fastest:
//
//   byte(r, c) = ((r/8) * (C/8) + c/8) * 128 + (r%8) * 16 + (c%8) * 2
//
// so core matrices adjacent along the columns are 128 B apart and row groups
// are C*16 B apart.  The same bytes serve two roles:
//   * K-major operand (rows = M or N, columns = K), sdesc_k: leading byte
//     offset = 128 (next core matrix along K), stride byte offset = C*16
//     (next 8-row group along M/N);
//   * MN-major operand (rows = K, columns = M or N), sdesc_mn: leading byte
//     offset = C*16 (next 8-row group along K), stride byte offset = 128
//     (next core matrix along M/N).
// Both assignments were checked against a CPU GEMM for every operand shape
// used here (tests/test_gpu_farfield.py::test_tcgen05_gemm).  A row-major
// activation tile written once per thread row therefore feeds the forward
// GEMM (K-major A) and the weight-gradient GEMM (MN-major A and B)
// unchanged.
//
// Accumulators live in tensor memory (TMEM): for M = 128 with cta_group::1,
// row i of D is TMEM lane i and column j is TMEM column base + j (FP32).
// Warp w of the CTA may read lanes 32(w%4) .. 32(w%4)+31.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace lpm {
namespace tc {

__device__ __forceinline__ uint32_t cm_off(int r, int c, int ncols) {
  return (uint32_t)((((r >> 3) * (ncols >> 3) + (c >> 3)) << 7) + ((r & 7) << 4) +
                    ((c & 7) << 1));
}

// Shared-memory matrix descriptor (tcgen05), no swizzle: start address,
// leading / stride byte offsets (all >> 4), fixed constant 0b001 at bit 46.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Descriptors of a tile with `cols` bf16 columns in the layout above.
__device__ __forceinline__ uint64_t sdesc_k(uint32_t saddr, int cols) {
  return sdesc(saddr, 128u, uint32_t(cols) * 16u);
}
__device__ __forceinline__ uint64_t sdesc_mn(uint32_t saddr, int cols) {
  return sdesc(saddr, uint32_t(cols) * 16u, 128u);
}

// Instruction descriptor for kind::f16 with BF16 A/B and FP32 D.
// a_mn / b_mn select MN-major operands (transpose bits 15 / 16).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
         ((b_mn ? 1u : 0u) << 16) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive (once) on the mbarrier when every MMA this thread issued completes.
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          (uint32_t)__cvta_generic_to_shared(bar))
      : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes -> visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_smem_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Warp-collective TMEM allocation (ncols a power of two >= 32); the base
// address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Split form of ld16 for software pipelining: ld16_issue starts the load,
// ld16_wait waits for every load of this thread and ties the registers to the
// wait, so no use of them can be scheduled before it.
__device__ __forceinline__ void ld16_issue(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void ld16_wait(uint32_t* r) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

// TMEM address of (lane base of this warp, column c).
__device__ __forceinline__ uint32_t lane_addr(uint32_t tbase, int warp, int col) {
  return tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)col;
}

// Pack two floats into a bf16x2 word (round to nearest even).
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

}  // namespace tc
}  // namespace lpm

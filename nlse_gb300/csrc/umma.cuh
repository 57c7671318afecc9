// Fifth-generation tensor-core (tcgen05) helpers for sm_103a in inline PTX:
// tensor-memory (TMEM) allocation, BF16 x BF16 -> FP32 matrix multiply with
// the accumulator in TMEM, completion through an mbarrier, and TMEM -> register
// loads.  One CTA (cta_group::1), operands in shared memory in the canonical
// K-major layout without swizzle.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "tma.cuh"

namespace nlse {

// ---- operand layout ---------------------------------------------------------
// An R x K tile of BF16 (R rows, K contiguous elements per row in the logical
// matrix) is stored as 8 x 8 "core matrices" of 8 rows x 16 bytes each; core
// matrix (r/8, k/8) starts at byte (r/8)*SBO + (k/8)*LBO and its row r%8 at
// +16*(r%8).  Here the K-adjacent core matrices are packed (LBO = 128 bytes)
// and the 8-row groups follow each other (SBO = 16*K bytes).
constexpr uint32_t kUmmaLbo = 128;
__host__ __device__ constexpr uint32_t umma_sbo(int K) { return 16u * (uint32_t)K; }

// Element index of (r, k) in such a tile.
__host__ __device__ constexpr int umma_off(int r, int k, int K) {
  return (r >> 3) * (8 * K) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N (M in {64, 128}, N a multiple of 16 up to 256).
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// D (TMEM) [+]= A * B^T for one K = 16 slice; issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on `bar` once every MMA this thread issued so far has completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(bar))
      : "memory");
}

// ---- tensor memory ---------------------------------------------------------
// Allocation (whole warp): the TMEM address is written to *dst (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_addr(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane (warp w of a
// four-warp group reads lanes 32*(w%4) .. 32*(w%4)+31).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// TMEM address of lane block (warp % 4) and column `col` from the allocated base.
__device__ __forceinline__ uint32_t tmem_lane_addr(uint32_t base, int warp, int col) {
  return base + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)col;
}

}  // namespace nlse

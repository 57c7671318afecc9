// Bulk-copy (TMA) and mbarrier helpers in inline PTX for sm_103a, with
// time-bounded waits.
#pragma once
#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>
#include <stdint.h>

namespace nlse {

// Error codes a kernel may record in the plan's status word.
enum : int { DEV_OK = 0, DEV_WAIT_TIMEOUT = 1, DEV_SMEM_MISALIGNED = 2 };

// A wait gives up after this many nanoseconds of the global timer.
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Make the initialised barriers visible to the async (bulk-copy) proxy.
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses before
// later bulk copies into the same shared memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Polls after which a wait gives up even if the timer should not advance
// (each poll is a try_wait, which may itself suspend for a while).
constexpr unsigned kWaitMaxPolls = 1u << 26;

// Whether a kernel's dynamic shared memory starts on the 128-byte boundary
// its tensor-map copies need (every thread; the caller records a failure
// and returns before issuing any copy when it does not).
__device__ __forceinline__ bool smem_base_aligned(const void* p) { return (smem_addr(p) & 127u) == 0; }

// Wait for phase `parity` of the barrier; false if limit_ns passed first.
__device__ __forceinline__ bool mbar_wait_limit(uint64_t* bar, unsigned parity,
                                                unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned n = 0; !mbar_try_wait(bar, parity); ++n)
    if (global_ns() - t0 > limit_ns || n > kWaitMaxPolls) return false;
  return true;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  return mbar_wait_limit(bar, parity, kWaitLimitNs);
}

// Contiguous global -> shared bulk copy completing on `bar` (sizes and both
// addresses multiples of 16 bytes).
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src_gmem, unsigned bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst_smem)), "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// 4-D tiled tensor-map store of a shared-memory box (128-byte aligned source)
// into global memory, in the calling thread's bulk group.  The box's shared
// writes must be fenced (fence_proxy_async_smem by every writer, then a
// barrier) before the store is issued.
__device__ __forceinline__ void tensor_store_4d(const CUtensorMap* map, int c0, int c1, int c2,
                                                int c3, const void* src_smem) {
  asm volatile(
      "cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(src_smem))
      : "memory");
}
__device__ __forceinline__ void bulk_commit_group() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// every committed store of this thread has finished reading shared memory
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// every committed store of this thread is complete in global memory
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Bring `bytes` of global memory into L2 ahead of their loads (no completion
// to wait for).  src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src_gmem, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src_gmem), "r"(bytes) : "memory");
}

// 4-D tiled tensor-map load into shared memory completing on `bar`; the map
// lives in kernel parameter space (__grid_constant__).  Coordinate c0 (the
// innermost) must be a multiple of 16 bytes; it is always 0 here.
__device__ __forceinline__ void tensor_load_4d(void* dst_smem, const CUtensorMap* map, int c0,
                                               int c1, int c2, int c3, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst_smem)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(smem_addr(bar))
      : "memory");
}

}  // namespace nlse

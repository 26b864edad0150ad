// Asynchronous bulk copies (TMA) and shared-memory mbarriers, sm_90+ PTX.
//
// Every wait is bounded: mbar_wait() gives up after `max_tries` polls and
// reports it, so a copy that never lands turns into an error status instead
// of a hung kernel.  Callers make the give-up decision block-uniform
// (__syncthreads_or) before leaving.
#pragma once
#include <cuda.h>  // CUtensorMap (type only; the encoder is fetched through the runtime)
#include <cuda_runtime.h>
#include <stdint.h>

namespace lgx {

// Polls of one bounded mbarrier wait (each poll may suspend the thread for a
// hardware-chosen interval): far above any copy's latency, far below a hang.
constexpr int kMbarMaxTries = 1 << 22;

// Device status word values written by the streamed kernels.
constexpr int kStatusCopyTimeout = 1;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Retire an mbarrier before its shared memory is used for anything else.
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Make mbarrier initialisation and earlier generic-proxy shared-memory
// accesses visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for phase `parity` of `bar` to complete; false if it did not within
// `max_tries` polls (kMbarMaxTries by default).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int max_tries = kMbarMaxTries) {
  for (int i = 0; i < max_tries; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 2D tiled tensor load of one box into shared memory, completing on `bar`.
// x is the innermost coordinate (elements), y the row.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Contiguous bulk copy global -> shared (both 16-byte aligned, bytes % 16 == 0).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// 2D tiled tensor store of one box from shared memory (bulk-group
// completion; x aligned like a load, x and y non-negative).  The writing
// threads fence their shared stores to the async proxy and meet at a barrier
// before one thread issues it.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// every committed store has finished reading its shared-memory source
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// every committed store has completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Bulk prefetch of [src, src + bytes) into L2; nothing to wait for.  A
// source that is not 16-byte aligned is skipped (a hint only), the size
// rounded down to whole 16-byte units.
__device__ __forceinline__ void prefetch_l2(const void* src, unsigned bytes) {
  bytes &= ~15u;
  if ((reinterpret_cast<uintptr_t>(src) & 15u) != 0 || bytes == 0) return;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(reinterpret_cast<uint64_t>(src)), "r"(bytes)
               : "memory");
}

// Byte offset of 16-byte chunk `chunk` (0..7) of row `row` in a box loaded
// with CU_TENSOR_MAP_SWIZZLE_128B (128-byte rows, box base 1024-aligned).
__device__ __forceinline__ int swz128(int row, int chunk) { return row * 128 + ((chunk ^ (row & 7)) << 4); }

}  // namespace lgx

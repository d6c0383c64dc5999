// Tensor-memory-accelerator (TMA) and mbarrier building blocks for the
// force kernels, written as inline PTX for sm_103a.
//
// Every wait on an mbarrier is bounded: after kMaxWaitTries polls the
// waiting thread records GFMD_ETIMEDOUT in the handle's device error word and
// the kernel gives up on that tile instead of spinning forever.
#ifndef GFMD_GB300_TMA_CUH
#define GFMD_GB300_TMA_CUH

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace gfmd {

// Polls of an mbarrier before a wait is declared lost (each poll may suspend
// the thread for a hardware-defined interval; ~2^24 polls is seconds).
constexpr unsigned kMaxWaitTries = 1u << 24;

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisations visible to the async proxy (TMA).
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Arrive on the barrier and announce `bytes` of transaction count.
__device__ __forceinline__ void mbar_arrive_tx(uint64_t *bar, unsigned bytes) {
  asm volatile(
      "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

// Waits until the barrier's phase `parity` completed; false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  const unsigned a = smem_addr(bar);
  for (unsigned it = 0; it < kMaxWaitTries; it++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 3-D tiled TMA load global -> shared, completion counted on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
          smem_addr(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}

// 3-D tiled TMA store shared -> global (bulk-group completion).
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, int c0, int c1, int c2, const void *src) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(map), "r"(c0),
      "r"(c1), "r"(c2), "r"(smem_addr(src))
      : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }

// Wait until at most N committed bulk groups still read shared memory.
template <int N> __device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
template <int N> __device__ __forceinline__ void bulk_wait() {
  asm volatile("cp.async.bulk.wait_group %0;\n" ::"n"(N) : "memory");
}

// Orders this thread's generic-proxy shared-memory writes before later
// async-proxy (TMA) reads of them.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];\n" ::"l"(map) : "memory");
}

// Asynchronous prefetch of `bytes` (a multiple of 16) of global memory from
// the 16-byte-aligned address g into L2.
__device__ __forceinline__ void bulk_prefetch_l2(const void *g, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(g), "r"(bytes) : "memory");
}

}  // namespace gfmd

#endif

// async_copy.cuh -- mbarrier waits and bulk (TMA) copies into shared memory,
// shared by the TMA-fed tile kernel (tile_tma.cuh) and the row reductions
// (reduce.cu).  Every wait is bounded: a copy that has not landed after
// TMA_WAIT_NS makes the caller set PHCU_ST_TIMEOUT instead of spinning on.
#pragma once

#include <stdint.h>

namespace phcu {

constexpr uint64_t TMA_WAIT_NS = 1000000000ull;  // give up on a copy after 1 s

__device__ __forceinline__ uint64_t tma_now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// try_wait suspends the thread for up to the hinted 2 us while the phase is
// incomplete, so waiting warps do not spin on the issue slots.
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(2000u)
      : "memory");
  return ok != 0;
}
// Waits for the phase with the given parity to complete; false after limit_ns.
static __device__ __noinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = tma_now_ns();
  for (;;) {
    for (int i = 0; i < 32; i++)
      if (mbar_try_wait(bar, parity)) return true;
    if (tma_now_ns() - t0 > limit_ns) return false;
  }
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One contiguous run of `bytes` (a multiple of 16, both addresses 16-byte
// aligned) from global into shared memory, completing on bar.
__device__ __forceinline__ void bulk_load_1d(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

}  // namespace phcu

// Bulk (TMA) copies global -> shared completed on an mbarrier, and the bounded wait on
// it (device side; used by the tree preconditioner and the tiled explicit step).
#pragma once
#include <stdint.h>

namespace nrt {

// ---- bulk (TMA) copies global -> shared, completed on an mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Asks for bytes [p, p + bytes) to be brought into L2 (no completion, no data returned);
// 16-byte aligned address and size, like the bulk copies.
__device__ __forceinline__ void prefetch_l2(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
// One arrival on an mbarrier (a consumer releasing a buffer).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Orders this thread's earlier generic-proxy accesses before later bulk (async-proxy) ones.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async;" ::: "memory");
}

// Waits for phase `phase` of the tile barrier; gives up after about two seconds of
// clock (the copies it waits for are in bounds and always land, so giving up means a
// device fault), raising the error word the host checks.
__device__ __forceinline__ void mbar_wait(uint64_t *bar, uint32_t phase, int *err) {
  if (mbar_try_wait(bar, phase)) return;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, phase)) {
    if (clock64() - t0 > 4000000000ll) {
      atomicOr(err, 1);
      return;
    }
  }
}

// As mbar_wait, and says whether the phase completed.
__device__ __forceinline__ bool mbar_wait_ok(uint64_t *bar, uint32_t phase, int *err) {
  if (mbar_try_wait(bar, phase)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, phase)) {
    if (clock64() - t0 > 4000000000ll) {
      atomicOr(err, 1);
      return false;
    }
  }
  return true;
}

}  // namespace nrt

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

// Bytes of the bulk copy of elements [o, o + n) of an array (16-byte aligned base): the
// window rounded out to 16-byte boundaries.
template <typename X>
__device__ __forceinline__ uint32_t stage_bytes(int64_t o, int64_t n) {
  const uint64_t lo = ((uint64_t)o * sizeof(X)) & ~(uint64_t)15;
  const uint64_t hi = ((uint64_t)(o + n) * sizeof(X) + 15) & ~(uint64_t)15;
  return (uint32_t)(hi - lo);
}
template <typename X>
__device__ __forceinline__ void stage(unsigned char *dst, const X *a, int64_t o, int64_t n,
                                      uint64_t *bar) {
  const uint64_t lo = ((uint64_t)o * sizeof(X)) & ~(uint64_t)15;
  bulk_load(dst, (const char *)a + lo, stage_bytes<X>(o, n), bar);
}
// The shared-memory copy of element o of a staged array.
template <typename X>
__device__ __forceinline__ const X *staged(const unsigned char *dst, int64_t o) {
  return (const X *)(dst + (((uint64_t)o * sizeof(X)) & 15));
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

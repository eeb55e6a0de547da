// spx_tma.cuh — bulk asynchronous copies (global -> shared) completed on an
// mbarrier, for staging contiguous ranges of stage vectors while a CTA computes.
//
// Usage (one phase per barrier per launch): thread 0 calls mbar_init, then
// fence_mbar_init; the CTA synchronises; thread 0 arms the barrier with the
// total byte count (mbar_arm) and issues the copies (bulk_g2s); consumers wait
// with mbar_wait_bounded on parity 0.  Every copy needs 16-byte aligned
// addresses and a size that is a multiple of 16 bytes (always true for whole
// complex128 entries of a 16-byte aligned vector).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace spx {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make initialised barriers visible to the asynchronous (bulk copy) proxy
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one arrival that also announces `bytes` of transactions to come
__device__ __forceinline__ void mbar_arm(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// invalidate a barrier whose phases are all complete, so it can be initialised again
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// order this thread's earlier generic-proxy view of memory (including data other
// CTAs published and this thread acquired) before its later bulk copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait until *p >= target (wrap-free counters), giving up after `limit` polls.
__device__ __forceinline__ bool wait_counter(const unsigned int* p, unsigned int target, int limit = 1 << 22) {
  for (int i = 0; i < limit; ++i) {
    if (ld_acquire_u32(p) >= target) return true;
    __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
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

// Wait for phase `parity` to complete, giving up after `limit` polls (each
// poll may suspend the thread for a short, hardware-defined time).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit = 1 << 22) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

}  // namespace spx

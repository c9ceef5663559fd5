// tma.cuh -- inline-PTX helpers for 1-D bulk TMA copies (cp.async.bulk) completed on
// shared-memory mbarriers, with bounded waits.
#pragma once
#include <stdint.h>

namespace pog {

// Device-side error word: bit 0 = an mbarrier wait gave up (bounded spin exceeded).  Read and
// cleared by pog_device_status().  Defined here: lbm_tma.cu is the only translation unit that
// includes this header.
__device__ unsigned int g_device_error = 0u;
constexpr unsigned int DEV_ERR_WAIT_TIMEOUT = 1u;
// try_wait already suspends for a hardware time slice per poll; 2^21 polls is well above a
// second, far beyond any real copy latency.
constexpr uint32_t MBAR_SPIN_LIMIT = 1u << 21;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared; dst/src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.  Returns false (and raises
// the device error word) when the spin limit is exceeded.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < MBAR_SPIN_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(&g_device_error, DEV_ERR_WAIT_TIMEOUT);
  return false;
}

}  // namespace pog

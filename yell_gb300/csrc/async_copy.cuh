// Asynchronous copies into shared memory for sm_103a: bulk copies whose
// completion is counted on an mbarrier, and bounded waits on that mbarrier.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace yell_gb300 {

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(mbar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Announces `bytes` of copies on the mbarrier (one arrival).
__device__ __forceinline__ void mbar_expect(uint64_t* mbar, uint32_t bytes) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(mbar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

// Shared memory read through the generic proxy is about to be written by the
// async proxy (a copy into a buffer the CTA has finished reading).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(mbar);
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(d), "l"(src), "r"(bytes), "r"(b) : "memory");
}

// Waits for phase `parity` of the mbarrier for at most timeout_ns of the
// global timer (1 s unless given) or 2^24 polls.  When either limit runs out
// it records `timeout_code` in *status (if still 0) and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t* status,
                                          uint32_t timeout_code, uint64_t timeout_ns = 1000000000ull) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(mbar);
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t i = 0; i < (1u << 24); ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 255u) == 255u && globaltimer_ns() - t0 > timeout_ns) break;
  }
  if (status) atomicCAS(status, 0u, timeout_code);
  return false;
}

}  // namespace yell_gb300

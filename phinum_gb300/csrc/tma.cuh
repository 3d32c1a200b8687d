// Inline-PTX helpers for bulk asynchronous copies (TMA engine, 1-D bulk form)
// and shared-memory mbarriers, sm_90+ (used on sm_103a).
//
// Every wait is bounded: after kWaitPolls polls the waiter records an error
// code and gives up, so a broken pipeline ends the kernel with an error
// status instead of hanging the GPU.
#pragma once

#include <stdint.h>

namespace phn {

constexpr long long kWaitPolls = 20000000LL;  // with backoff: several seconds

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits until the phase with the given parity has completed.  Returns false
// if it does not within the poll budget (then `code` goes to *err and the
// block-wide *abort flag is raised) or if another thread of the block raised
// *abort meanwhile.  err and abort may be null.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int *err, int code, int *abort,
                                          long long polls = kWaitPolls) {
  volatile int *ab = abort;
  for (long long i = 0; i < polls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (ab && *ab) return false;
    if (i > 32) __nanosleep(64);
  }
  if (ab) *ab = 1;
  if (err) atomicExch(err, code);
  return false;
}

// 1-D bulk copy global -> shared, completing `bytes` on the mbarrier.
// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

}  // namespace phn

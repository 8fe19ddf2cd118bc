// nb_tma.cuh -- bulk (TMA) copies into shared memory with an mbarrier, and
// the device error flag that bounded waits report through.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nb {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// One contiguous global -> shared copy of `bytes` (multiple of 16, both
// addresses 16-byte aligned), completion counted on bar.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Asks the TMA unit to bring `bytes` (a multiple of 16, src 16-byte
// aligned) into L2 ahead of use; there is no completion to wait for.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of bar; gives up after `limit` polls (each poll
// suspends in hardware for a bounded time), sets bit 0 of *err (the
// library's device error word, read by device_error_check) and returns false.
constexpr unsigned kWaitPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity,
                                                  unsigned *err,
                                                  unsigned limit = kWaitPolls) {
  for (unsigned it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicOr(err, 1u);
  return false;
}

// ------------------------------------------- element block by bulk copy --
// An element kernel's one bulk copy of `bytes` into shared memory (thread 0
// calls the first function when the CTA starts; bar is fresh, phase 0).
// wait_test (the library's timeout self-test, nb_set_wait_test): the
// barrier expects 16 bytes more than the copy brings, so the wait below runs
// out for certain.
__device__ __forceinline__ void block_copy_begin(uint64_t *bar, void *dst, const void *src,
                                                 unsigned bytes, int wait_test) {
  mbar_init(bar, 1);
  mbar_arrive_expect_tx(bar, bytes + (wait_test ? 16u : 0u));
  bulk_g2s(dst, src, bytes, bar);
}

// Every thread of the CTA calls this before it reads the copied block.
// Returns true when the copy has landed.  When any thread's wait ran out
// (the error word is then set), the CTA agrees on it, lets its copy land
// (one more bounded wait; in the self-test a 16-byte copy from src16 into
// pad16 first completes the phase) and gets false: the caller then skips
// the element's arithmetic and stores and returns, its results invalid.
__device__ __forceinline__ bool block_copy_wait(uint64_t *bar, unsigned *err, int wait_test,
                                                void *pad16, const void *src16) {
  const bool mine = mbar_wait_bounded(bar, 0, err, wait_test ? 64u : kWaitPolls);
  if (__syncthreads_and(mine ? 1 : 0)) return true;
  if (wait_test && threadIdx.x == 0 && threadIdx.y == 0) bulk_g2s(pad16, src16, 16u, bar);
  mbar_wait_bounded(bar, 0, err);
  __syncthreads();
  return false;
}

}  // namespace nb

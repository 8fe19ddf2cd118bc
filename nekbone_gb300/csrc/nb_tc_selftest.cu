// nb_tc_selftest.cu -- one tcgen05 MMA on known small-integer operands, used
// by the tests to check the tensor-core building blocks (descriptor bit
// layouts, operand layout, tensor-memory lane/column mapping) before the
// tensor-core operator relies on them.  All shared-memory addresses lie in
// the two tiles; the completion wait is bounded; tensor memory is always
// released.
#include <cuda_bf16.h>

#include "../../include/nekbone_gb300.h"
#include "nb_internal.h"
#include "nb_tc.cuh"

namespace nb {
namespace {

__host__ __device__ inline int tc_a(int r, int k) { return ((r * 7 + k * 3) % 13) - 6; }
__host__ __device__ inline int tc_b(int n, int k) { return ((n * 5 + k * 11) % 9) - 4; }

// The tiles sit in a 200 KB dynamic shared buffer, A at 0 and B at 128 KB,
// so that even a misread descriptor field would keep the tensor core's reads
// inside this CTA's own allocation.
constexpr size_t kSelftestSmem = 200 * 1024;

template <bool BF16>
__global__ void __launch_bounds__(128) k_tc_selftest(float *out, unsigned *err) {
  extern __shared__ __align__(1024) unsigned char dyn[];
  unsigned char *A = dyn;
  unsigned char *B = dyn + 128 * 1024;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t slot;
  const int t = threadIdx.x, w = t >> 5;
  for (int k = 0; k < 16; ++k) {
    if (BF16)
      *reinterpret_cast<__nv_bfloat16 *>(A + tc::kmajor16_offset(t, k)) =
          __int2bfloat16_rn(tc_a(t, k));
    else
      *reinterpret_cast<__half *>(A + tc::kmajor16_offset(t, k)) = __int2half_rn(tc_a(t, k));
  }
  if (t < 16)
    for (int k = 0; k < 16; ++k) {
      if (BF16)
        *reinterpret_cast<__nv_bfloat16 *>(B + tc::kmajor16_offset(t, k)) =
            __int2bfloat16_rn(tc_b(t, k));
      else
        *reinterpret_cast<__half *>(B + tc::kmajor16_offset(t, k)) = __int2half_rn(tc_b(t, k));
    }
  tc::fence_smem_to_async();
  if (t == 0) mbar_init(&bar, 1);
  if (w == 0) {
    tc::tmem_alloc(&slot, 32);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = slot;
  if (t == 0) {
    tc::mma_f16(taddr, tc::smem_desc(A, 128, 256), tc::smem_desc(B, 128, 256),
                tc::idesc_f16(128, 16, BF16), false);
    tc::mma_commit(&bar);
  }
  const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bar, 0, err));
  tc::fence_after_sync();
  float v[16];
  if (ok) {
    tc::tmem_ld16(taddr + (uint32_t(32 * w) << 16), v);
  } else {
    for (int c = 0; c < 16; ++c) v[c] = 0.f;
  }
  for (int c = 0; c < 16; ++c) out[t * 16 + c] = v[c];
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(taddr, 32);
}

}  // namespace
}  // namespace nb

using namespace nb;

// Runs the tcgen05 self-test (bf16 != 0: BF16 operands, else F16); returns
// the number of the 128x16 results that differ from the exact product.
extern "C" int nb_tc_selftest(int bf16, int *mismatches) {
  clear_status();
  float *d = nullptr;
  NB_CUDA(cudaMalloc(&d, 128 * 16 * sizeof(float)));
  unsigned *err = device_error_word();
  NB_CUDA(cudaFuncSetAttribute(k_tc_selftest<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(kSelftestSmem)));
  NB_CUDA(cudaFuncSetAttribute(k_tc_selftest<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(kSelftestSmem)));
  if (bf16)
    k_tc_selftest<true><<<1, 128, kSelftestSmem>>>(d, err);
  else
    k_tc_selftest<false><<<1, 128, kSelftestSmem>>>(d, err);
  NB_CUDA(cudaGetLastError());
  float h[128 * 16];
  NB_CUDA(cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost));
  cudaFree(d);
  NB_TRY(device_error_check(0));
  int bad = 0;
  for (int r = 0; r < 128; ++r)
    for (int n = 0; n < 16; ++n) {
      int ref = 0;
      for (int k = 0; k < 16; ++k) ref += tc_a(r, k) * tc_b(n, k);
      if (h[r * 16 + n] != float(ref)) ++bad;
    }
  *mismatches = bad;
  return NB_OK;
}

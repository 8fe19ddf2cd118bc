// nb_tc.cuh -- fifth-generation tensor core (tcgen05) building blocks for
// sm_103a: tensor-memory allocation, shared-memory matrix descriptors, the
// instruction descriptor of kind::f16 MMAs, MMA issue and commit, and
// tensor-memory loads.  Written from the PTX ISA's tcgen05 description.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "nb_tma.cuh"

namespace nb {
namespace tc {

// ---- shared-memory matrix descriptor (64 bit) -------------------------------
// bits  0-13  start address >> 4      bits 16-29  leading byte offset >> 4
// bits 32-45  stride byte offset >> 4 bits 46-47  version (1)
// bits 49-51  base offset (0)         bit 52      LBO mode (0)
// bits 61-63  swizzle (0 = none)
// Canonical K-major layout without swizzle: 8x8 "core matrices" of 8 rows x
// 16 bytes, 128 contiguous bytes each; LBO = byte distance between core
// matrices adjacent along K, SBO = between core matrices adjacent along M/N.
__device__ __forceinline__ uint64_t smem_desc(const void *base, uint32_t lbo, uint32_t sbo) {
  const uint32_t a = smem_u32(base);
  uint64_t d = 0;
  d |= uint64_t((a & 0x3FFFFu) >> 4);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// Byte offset of element (row, k), k < 16, in a K-major 16-wide tile laid out
// as above with LBO = 128 and SBO = 256 (2-byte elements).
__host__ __device__ __forceinline__ uint32_t kmajor16_offset(int row, int k) {
  return uint32_t((row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// ---- instruction descriptor, kind::f16 (32 bit) -----------------------------
// bits 4-5 D format (1 = F32), 7-9 A format, 10-12 B format (0 = F16,
// 1 = BF16), 15/16 A/B major (0 = K-major), 17-22 N >> 3, 24-28 M >> 4.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, bool bf16) {
  return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) |
         (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// ---- tensor memory ----------------------------------------------------------
// Warp-wide: allocates ncols (power of two >= 32) columns, writes the base
// address to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A * B^T for one M x N x 16 block; single thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}
// arrive on bar when every MMA issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive 32-bit columns of this thread's lane (warp w reads lanes
// 32(w%4) .. +31): taddr must carry the warp's lane base in bits 16-31.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%"
      "14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

}  // namespace tc
}  // namespace nb

// nb_ax_tc.cu -- the FP32 element operator with its six derivative
// contractions (local_grad3 and local_grad3_t, cg.f:170-212) on the
// tcgen05 tensor cores.
//
// Each 1-D line of the element -- lx1 values along the contracted index,
// e.g. u(0..lx1-1, j, k) for the r derivative -- is one row of a K-major
// 16-wide operand tile (128 rows per tile, K zero-padded to 16).  The row is
// scaled by a power of two to unit maximum (exact), then split into FP16
// hi = fp16(v) and lo = fp16(v - hi); D (or D^T) is split the same way.
// Three kind::f16 MMAs per tile, hi*hi + hi*lo + lo*hi, accumulate in FP32
// in tensor memory, which carries ~22 significant bits: the result matches
// an FP32 evaluation to rounding (lo*lo, ~2^-22 of the row maximum, is
// dropped).  Rows are unscaled when read back.  The metric step (cg.f:156-163)
// and the sum (tr + ts) + tt run on CUDA cores in FP32.
//
// One CTA (one warpgroup, 128 threads) per element, looping over elements;
// thread t owns row t of every tile.  Tensor memory: 16 columns per tile.
#include <cuda_fp16.h>

#include <algorithm>

#include "../../include/nekbone_gb300.h"
#include "nb_solver.h"
#include "nb_tc.cuh"

namespace nb {

namespace {

template <int LX>
struct TcCfg {
  static constexpr int L2 = LX * LX, L3 = LX * LX * LX;
  static constexpr int P = LX + 1;           // padded pitch along j
  static constexpr int PN = P * LX * LX;     // padded point array length
  static constexpr int T = (L2 + 127) / 128; // tiles per direction
  static constexpr int NT = 3 * T;           // tiles per phase
  static constexpr int COLS = NT * 16 <= 32 ? 32 : NT * 16 <= 64 ? 64 : NT * 16 <= 128 ? 128 : 256;
};

template <int LX>
struct TcShared {
  alignas(128) unsigned char A[TcCfg<LX>::NT][2][4096];   // [tile][hi,lo]
  alignas(128) unsigned char Bf[2][512];                  // D   split (hi, lo)
  alignas(128) unsigned char Bt[2][512];                  // D^T split
  float U[TcCfg<LX>::PN];
  float X[3][TcCfg<LX>::PN];   // ur/us/ut -> wr/ws/wt -> tr/ts/tt
  float scale[TcCfg<LX>::NT][128];
  alignas(8) uint64_t bar;
  uint32_t slot;
};

template <int LX>
__device__ __forceinline__ int pidx(int i, int j, int k) {
  return i + (LX + 1) * j + (LX + 1) * LX * k;
}

// element of line `lam` of direction d (0: r, 1: s, 2: t), position m
template <int LX>
__device__ __forceinline__ int line_point(int d, int lam, int m) {
  const int a = lam % LX, b = lam / LX;
  return d == 0 ? pidx<LX>(m, a, b) : d == 1 ? pidx<LX>(a, m, b) : pidx<LX>(a, b, m);
}

__device__ __forceinline__ void split_store(unsigned char *hi, unsigned char *lo, int row, int k,
                                            float v) {
  const __half h = __float2half_rn(v);
  const __half l = __float2half_rn(v - __half2float(h));
  *reinterpret_cast<__half *>(hi + tc::kmajor16_offset(row, k)) = h;
  *reinterpret_cast<__half *>(lo + tc::kmajor16_offset(row, k)) = l;
}

// Builds this thread's row of every tile from the point array of direction d,
// src + d * dstride, and records the row scale.
template <int LX>
__device__ __forceinline__ void build_rows(TcShared<LX> &sm, const float *src, int dstride) {
  typedef TcCfg<LX> C;
  const int t = threadIdx.x;
#pragma unroll 1
  for (int d = 0; d < 3; ++d)
#pragma unroll 1
    for (int tau = 0; tau < C::T; ++tau) {
      const int lam = tau * 128 + t, tile = d * C::T + tau;
      unsigned char *hi = sm.A[tile][0], *lo = sm.A[tile][1];
      float v[16];
      float mx = 0.f;
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        v[m] = (lam < C::L2 && m < LX) ? src[d * dstride + line_point<LX>(d, lam, m)] : 0.f;
        mx = fmaxf(mx, fabsf(v[m]));
      }
      int ex = 0;
      if (mx > 0.f) frexpf(mx, &ex);
      const float sdown = ldexpf(1.f, -ex);
      sm.scale[tile][t] = ldexpf(1.f, ex);
#pragma unroll
      for (int m = 0; m < 16; ++m) split_store(hi, lo, t, m, v[m] * sdown);
    }
}

// Thread 0: D[tile] = A_hi B_hi + A_hi B_lo + A_lo B_hi for every tile.
template <int LX>
__device__ __forceinline__ void issue_mmas(TcShared<LX> &sm, uint32_t tmem,
                                           unsigned char (*B)[512]) {
  typedef TcCfg<LX> C;
  const uint32_t idesc = tc::idesc_f16(128, 16, false);
  const uint64_t bhi = tc::smem_desc(B[0], 128, 256), blo = tc::smem_desc(B[1], 128, 256);
  for (int tile = 0; tile < C::NT; ++tile) {
    const uint32_t d = tmem + uint32_t(tile * 16);
    const uint64_t ahi = tc::smem_desc(sm.A[tile][0], 128, 256);
    const uint64_t alo = tc::smem_desc(sm.A[tile][1], 128, 256);
    tc::mma_f16(d, ahi, bhi, idesc, false);
    tc::mma_f16(d, ahi, blo, idesc, true);
    tc::mma_f16(d, alo, bhi, idesc, true);
  }
  tc::mma_commit(&sm.bar);
}

// Reads this thread's row of every tile back, unscales, scatters into X[d].
template <int LX>
__device__ __forceinline__ void drain_rows(TcShared<LX> &sm, uint32_t tmem) {
  typedef TcCfg<LX> C;
  const int t = threadIdx.x, w = t >> 5;
#pragma unroll 1
  for (int d = 0; d < 3; ++d)
#pragma unroll 1
    for (int tau = 0; tau < C::T; ++tau) {
      const int tile = d * C::T + tau, lam = tau * 128 + t;
      float y[16];
      tc::tmem_ld16(tmem + (uint32_t(32 * w) << 16) + uint32_t(tile * 16), y);
      if (lam < C::L2) {
        const float sc = sm.scale[tile][t];
#pragma unroll
        for (int m = 0; m < LX; ++m) sm.X[d][line_point<LX>(d, lam, m)] = y[m] * sc;
      }
    }
}

template <int LX>
__global__ void __launch_bounds__(128)
    k_ax_tc(float *__restrict__ w, const float *__restrict__ u, const float *__restrict__ g,
            const float *__restrict__ D, int nelt, unsigned *err) {
  typedef TcCfg<LX> C;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TcShared<LX> &sm = *reinterpret_cast<TcShared<LX> *>(smem_raw);
  const int t = threadIdx.x, wp = t >> 5;

  // split D and D^T once: Bf[n][m] = D(n,m), Bt[n][m] = D(m,n), zero padded
  for (int q = t; q < 256; q += 128) {
    const int n = q / 16, m = q % 16;
    const float df = (n < LX && m < LX) ? D[n + m * LX] : 0.f;
    const float dt = (n < LX && m < LX) ? D[m + n * LX] : 0.f;
    split_store(sm.Bf[0], sm.Bf[1], n, m, df);
    split_store(sm.Bt[0], sm.Bt[1], n, m, dt);
  }
  if (t == 0) mbar_init(&sm.bar, 1);
  if (wp == 0) {
    tc::tmem_alloc(&sm.slot, C::COLS);
    tc::tmem_relinquish();
  }
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.slot;
  unsigned phase = 0;
  bool healthy = true;

  for (int e = blockIdx.x; e < nelt; e += gridDim.x) {
    const size_t base = size_t(e) * C::L3;
    for (int q = t; q < C::L3; q += 128) {
      const int i = q % LX, j = (q / LX) % LX, k = q / C::L2;
      sm.U[pidx<LX>(i, j, k)] = u[base + q];
    }
    __syncthreads();
    // forward contractions: ur, us, ut (local_grad3)
    build_rows<LX>(sm, sm.U, 0);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (t == 0 && healthy) issue_mmas<LX>(sm, tmem, sm.Bf);
    healthy = __syncthreads_and(healthy ? mbar_wait_bounded(&sm.bar, phase, err) : 0) != 0;
    phase ^= 1u;
    tc::fence_after_sync();
    if (healthy) drain_rows<LX>(sm, tmem);
    tc::fence_before_sync();
    __syncthreads();
    // metric (cg.f:156-163), in place
    for (int q = t; q < C::L3; q += 128) {
      const int i = q % LX, j = (q / LX) % LX, k = q / C::L2;
      const int pq = pidx<LX>(i, j, k);
      const float ur = sm.X[0][pq], us = sm.X[1][pq], ut = sm.X[2][pq];
      const float2 *gp = reinterpret_cast<const float2 *>(g + 6 * (base + q));
      const float2 g01 = gp[0], g23 = gp[1], g45 = gp[2];
      float wr = mul_rn(g01.x, ur);
      wr = fma_rn(g01.y, us, wr);
      wr = fma_rn(g23.x, ut, wr);
      float ws = mul_rn(g01.y, ur);
      ws = fma_rn(g23.y, us, ws);
      ws = fma_rn(g45.x, ut, ws);
      float wt = mul_rn(g23.x, ur);
      wt = fma_rn(g45.x, us, wt);
      wt = fma_rn(g45.y, ut, wt);
      sm.X[0][pq] = wr;
      sm.X[1][pq] = ws;
      sm.X[2][pq] = wt;
    }
    __syncthreads();
    // transposed contractions: tr, ts, tt (local_grad3_t)
    build_rows<LX>(sm, sm.X[0], C::PN);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (t == 0 && healthy) issue_mmas<LX>(sm, tmem, sm.Bt);
    healthy = __syncthreads_and(healthy ? mbar_wait_bounded(&sm.bar, phase, err) : 0) != 0;
    phase ^= 1u;
    tc::fence_after_sync();
    if (healthy) drain_rows<LX>(sm, tmem);
    tc::fence_before_sync();
    __syncthreads();
    for (int q = t; q < C::L3; q += 128) {
      const int i = q % LX, j = (q / LX) % LX, k = q / C::L2;
      const int pq = pidx<LX>(i, j, k);
      w[base + q] = add_rn(add_rn(sm.X[0][pq], sm.X[1][pq]), sm.X[2][pq]);
    }
    __syncthreads();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (wp == 0) tc::tmem_dealloc(tmem, C::COLS);
}

template <int LX>
int launch_tc_lx(float *w, const float *u, const float *g, const float *D, int nelt,
                 cudaStream_t s) {
  const size_t sm = sizeof(TcShared<LX>);
  static bool attr_set = false;
  if (!attr_set) {
    NB_CUDA(cudaFuncSetAttribute(k_ax_tc<LX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(sm)));
    attr_set = true;
  }
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int grid = std::min(nelt, nsm * 2);
  k_ax_tc<LX><<<grid, 128, sm, s>>>(w, u, g, D, nelt, device_error_word());
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

}  // namespace

// w = A_L u (element products only) with tensor-core contractions
int launch_ax_tc(const Operator &op, float *w, const float *u, const float *g, cudaStream_t s) {
  switch (op.lx) {
#define NB_CASE(L) case L: return launch_tc_lx<L>(w, u, g, op.fD, op.nelt, s);
    NB_CASE(2) NB_CASE(3) NB_CASE(4) NB_CASE(5) NB_CASE(6) NB_CASE(7) NB_CASE(8)
    NB_CASE(9) NB_CASE(10) NB_CASE(11) NB_CASE(12) NB_CASE(13) NB_CASE(14) NB_CASE(15)
    NB_CASE(16)
#undef NB_CASE
    default:
      return fail(NB_ERR_UNSUPPORTED, "tensor-core ax: lx1=%d not supported", op.lx);
  }
}

// w = mask(QQ^T A_L u + 0.1 u) with the tensor-core element products
int apply_ax_tc(const Operator &op, float *w, const float *u, const float *g, cudaStream_t s) {
  NB_TRY(launch_ax_tc(op, w, u, g, s));
  NB_TRY(gs_exec(op.gs, w, 2, 1, 0, s));
  NB_TRY(vec_add2s2<float>(w, u, 0.1, op.n, s));
  return vec_mask<float>(w, op.d_mask_list, op.n_mask, s);
}

}  // namespace nb

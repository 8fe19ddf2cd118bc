// nb_probe.cu -- issue-rate probe of the pipes the element operators use:
// FP64 fused multiply-add (the even-odd FP64 operator's bound), 32x32->64
// integer multiply-add (the fixed-point operator's products), 32-bit integer
// add (its shifts, splits and conversions) and FP32 fused multiply-add.
// Every thread runs 8 independent chains; results are folded into one store
// per thread so nothing is optimised away.
#include "nb_internal.h"

namespace nb {
namespace {

constexpr int kChains = 8;

template <int OP>
__global__ void __launch_bounds__(256) k_pipe(unsigned long long *out, unsigned seed, int iters) {
  unsigned a[kChains];
  unsigned long long w[kChains];
  float f[kChains];
  double d[kChains];
  const unsigned t = threadIdx.x + blockIdx.x * blockDim.x;
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    a[c] = t * 7u + unsigned(c) + seed;
    w[c] = a[c];
    f[c] = float(a[c] & 1023u);
    d[c] = double(a[c]);
  }
  const unsigned b = seed | 1u;
  const float fb = 1.0001f, fc = 0.5f;
  const double db = 1.0000001, dc = 0.5;
#pragma unroll 1
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      if (OP == 0) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(d[c]) : "d"(db), "d"(dc));
      if (OP == 1) asm volatile("mad.wide.s32 %0, %1, %2, %0;" : "+l"(w[c]) : "r"(a[c]), "r"(b));
      if (OP == 2) asm volatile("add.s32 %0, %0, %1;" : "+r"(a[c]) : "r"(b));
      if (OP == 3) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(f[c]) : "f"(fb), "f"(fc));
    }
  }
  unsigned long long s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c)
    s += a[c] + w[c] + __float_as_uint(f[c]) + (unsigned long long)__double_as_longlong(d[c]);
  out[t] = s;
}

template <int OP>
int time_pipe(unsigned long long *out, int blocks, int iters, cudaStream_t s, double *rate) {
  k_pipe<OP><<<blocks, 256, 0, s>>>(out, 1u, iters);  // warm-up
  NB_CUDA(cudaGetLastError());
  cudaEvent_t e0, e1;
  NB_CUDA(cudaEventCreate(&e0));
  NB_CUDA(cudaEventCreate(&e1));
  NB_CUDA(cudaEventRecord(e0, s));
  for (int r = 0; r < 3; ++r) k_pipe<OP><<<blocks, 256, 0, s>>>(out, unsigned(r + 2), iters);
  NB_CUDA(cudaEventRecord(e1, s));
  NB_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  NB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *rate = 3.0 * blocks * 256.0 * kChains * iters / (double(ms) * 1e-3);
  return NB_OK;
}

}  // namespace
}  // namespace nb

// rates[0..3] = operations per second of DFMA, mad.wide.s32, 32-bit integer
// add and FFMA over the whole GPU (8 CTAs of 256 threads per SM; the FP64
// probe runs 1 CTA per SM with proportionally fewer iterations).
extern "C" int nb_pipe_rates(double *rates) {
  using namespace nb;
  clear_status();
  if (!rates) return fail(NB_ERR_ARG, "nb_pipe_rates: null output");
  int dev = 0, nsm = 0;
  NB_CUDA(cudaGetDevice(&dev));
  NB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = 8 * nsm;
  unsigned long long *out = nullptr;
  NB_CUDA(cudaMalloc(&out, sizeof(unsigned long long) * size_t(blocks) * 256));
  cudaStream_t s = nullptr;
  int st = time_pipe<0>(out, nsm, 2048, s, &rates[0]);
  if (!st) st = time_pipe<1>(out, blocks, 4096, s, &rates[1]);
  if (!st) st = time_pipe<2>(out, blocks, 4096, s, &rates[2]);
  if (!st) st = time_pipe<3>(out, blocks, 4096, s, &rates[3]);
  cudaFree(out);
  return st;
}

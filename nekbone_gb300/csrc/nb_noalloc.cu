// nb_noalloc.cu -- glsc3 on device vectors without any allocation.
//
// Who needs this: callers that cannot call cudaMalloc while the solver runs.
// Examples are a Fortran code whose device memory is owned by its own
// OpenACC / CUDA-Fortran pool, or a time-step loop that must not hit
// cudaMalloc's implicit device synchronisation.  The other entry points
// allocate their device buffers on first use.  This one keeps its only
// scratch -- the per-block partial sums and the last-block counter of the
// deterministic reduction -- in a fixed, file-scope device array.  Every GPU
// that loads the library holds that array until the process exits.
//
// Limits and sharing:
//  * n <= NB_NOALLOC_MAX_N: one partial per 4096 entries, at most 16384
//    partials (128 KiB of partials plus the counter).
//  * The array is shared by every call.  A call clears the counter it needs
//    before launching; the partials are written before they are read.
//    Calls that overlap on the GPU (different streams, no ordering between
//    them) race on the array and give wrong sums.
//  * The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current, and is the first
//    launch of the kernel.  Under lazy module loading (the default since
//    CUDA 12.2) that first launch loads the module, which can itself
//    allocate device memory and synchronise.  So make one warm-up call per
//    device before the region that must not allocate, and before any stream
//    capture begins.  The address cache is safe against concurrent first
//    calls from several host threads.
#include <atomic>

#include "../../include/nekbone_gb300.h"
#include "nb_internal.h"
#include "nb_kernels.cuh"

namespace nb {

namespace {

constexpr int kNoAllocMaxParts = 16384;
constexpr long kNoAllocPerBlock = 4096;  // entries reduced by one block
constexpr int kNoAllocThreads = 256;

// partials[kNoAllocMaxParts] doubles, then one unsigned counter
static __device__ __align__(256) unsigned char g_noalloc_scratch
    [kNoAllocMaxParts * sizeof(double) + 256];

constexpr int kMaxDevices = 64;
std::atomic<void *> g_scratch_ptr[kMaxDevices];  // zero-initialised (static storage)

__global__ void __launch_bounds__(kNoAllocThreads)
    k_glsc3_noalloc(const double *__restrict__ a, const double *__restrict__ b,
                    const double *__restrict__ m, long n, unsigned char *scratch,
                    double *result) {
  __shared__ double red[32];
  double *partial = reinterpret_cast<double *>(scratch);
  unsigned *counter = reinterpret_cast<unsigned *>(scratch + kNoAllocMaxParts * sizeof(double));
  const long lo = long(blockIdx.x) * kNoAllocPerBlock;
  const long hi = lo + kNoAllocPerBlock < n ? lo + kNoAllocPerBlock : n;
  double part = 0.0;
  for (long q = lo + threadIdx.x; q < hi; q += blockDim.x)
    part = fma_rn(mul_rn(a[q], b[q]), m[q], part);  // tmp + a*b*mult, math.f:613
  const double s = block_sum<double>(part, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block(counter, gridDim.x)) {
    const double v = block_sum_array(partial, gridDim.x, red);
    if (threadIdx.x == 0) *result = v;
  }
}

// Device address of the scratch array on the current device (set-up once).
int scratch_address(void **out) {
  int dev = 0;
  NB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(NB_ERR_UNSUPPORTED, "nb_glsc3_noalloc: device %d out of range", dev);
  void *p = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    // concurrent first calls may both look it up; they store the same address
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(NB_ERR_CUDA, "nb_glsc3_noalloc: cudaGetSymbolAddress: %s",
                  cudaGetErrorString(e));
    g_scratch_ptr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return NB_OK;
}

}  // namespace

}  // namespace nb

using namespace nb;

extern "C" int nb_glsc3_noalloc(const double *a, const double *b,
                                const double *mult, long n, double *result,
                                void *stream) {
  clear_status();
  if (n < 0 || n > NB_NOALLOC_MAX_N)
    return fail(NB_ERR_ARG,
                "nb_glsc3_noalloc: n=%ld outside 0..%ld (the fixed scratch holds "
                "%d partial sums of %ld entries each)",
                n, (long)NB_NOALLOC_MAX_N, kNoAllocMaxParts, kNoAllocPerBlock);
  if (!result || (n > 0 && (!a || !b || !mult)))
    return fail(NB_ERR_ARG, "nb_glsc3_noalloc: null device pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void *scr = nullptr;
  NB_TRY(scratch_address(&scr));
  unsigned char *base = static_cast<unsigned char *>(scr);
  // the counter must start at zero whatever the previous call left behind
  NB_CUDA(cudaMemsetAsync(base + kNoAllocMaxParts * sizeof(double), 0, sizeof(unsigned), s));
  if (n == 0) {
    NB_CUDA(cudaMemsetAsync(result, 0, sizeof(double), s));
    return NB_OK;
  }
  const int blocks = int((n + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
  k_glsc3_noalloc<<<blocks, kNoAllocThreads, 0, s>>>(a, b, mult, n, base, result);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

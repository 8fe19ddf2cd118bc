// nb_devflag.cu -- the library's device error word.  Kernels with bounded
// waits (bulk copies, barriers) set a bit in it when a wait runs out instead
// of hanging; the host checks it after solves.
#include "nb_internal.h"
#include "nb_tma.cuh"

namespace nb {

namespace {
unsigned *g_err = nullptr;
int g_wait_test = 0;
}

int wait_test_mode() { return g_wait_test; }

unsigned *device_error_word() {
  if (!g_err) {
    if (cudaMalloc(&g_err, sizeof(unsigned)) != cudaSuccess) {
      g_err = nullptr;
      return nullptr;
    }
    cudaMemset(g_err, 0, sizeof(unsigned));
  }
  return g_err;
}

// Fails with NB_ERR_CUDA when a kernel reported a wait that ran out (bit 0)
// or a fixed-point range check that failed (bit 1), and clears the word.
// Synchronises the stream.
int device_error_check(cudaStream_t s) {
  NB_CUDA(cudaStreamSynchronize(s));
  if (!g_err) return NB_OK;
  unsigned v = 0;
  NB_CUDA(cudaMemcpy(&v, g_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (v) {
    cudaMemset(g_err, 0, sizeof(unsigned));
    return fail(NB_ERR_CUDA, "%s (flags %u); results are invalid",
                (v & 1u) ? "a device-side wait timed out"
                         : "a fixed-point operator's range check failed",
                v);
  }
  return NB_OK;
}

}  // namespace nb

namespace nb {
cudaStream_t lib_stream();

namespace {
// One warp waits on an mbarrier that nothing arrives on, at most `polls`
// polls a thread: the bounded wait gives up, sets the error word and the
// kernel returns with nothing in flight.
__global__ void k_wait_selftest(unsigned polls, unsigned *err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  mbar_wait_bounded(&bar, 0, err, polls);
}
}  // namespace
}  // namespace nb

// The path every bounded wait takes when it runs out: the kernel returns,
// the host reads the error word and reports it, the context stays usable.
extern "C" int nb_wait_selftest(unsigned polls) {
  using namespace nb;
  clear_status();
  if (polls == 0 || polls > (1u << 16))
    return fail(NB_ERR_ARG, "nb_wait_selftest: polls=%u (1..65536)", polls);
  unsigned *err = device_error_word();
  if (!err) return fail(NB_ERR_CUDA, "nb_wait_selftest: no device error word");
  cudaStream_t s = lib_stream();
  NB_CUDA(cudaStreamSynchronize(s));
  k_wait_selftest<<<1, 32, 0, s>>>(polls, err);
  NB_CUDA(cudaGetLastError());
  return device_error_check(s);
}

// The same path in the real kernels: while on, every element kernel that
// brings its metric block in by a bulk copy sets its barrier to expect 16
// more bytes than the copy brings, so its bounded wait runs out; the CTA
// then lets the copy land, skips the element and sets the error word.
extern "C" int nb_set_wait_test(int on) {
  nb::clear_status();
  nb::g_wait_test = on != 0;
  return nb::NB_OK;
}

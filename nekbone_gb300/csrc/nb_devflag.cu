// nb_devflag.cu -- the library's device error word.  Kernels with bounded
// waits (bulk copies, barriers) set a bit in it when a wait runs out instead
// of hanging; the host checks it after solves.
#include "nb_internal.h"

namespace nb {

namespace {
unsigned *g_err = nullptr;
}

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

// Fails with NB_ERR_CUDA when a kernel reported a wait that ran out (and
// clears the word).  Synchronises the stream.
int device_error_check(cudaStream_t s) {
  NB_CUDA(cudaStreamSynchronize(s));
  if (!g_err) return NB_OK;
  unsigned v = 0;
  NB_CUDA(cudaMemcpy(&v, g_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (v) {
    cudaMemset(g_err, 0, sizeof(unsigned));
    return fail(NB_ERR_CUDA, "a device-side wait timed out (flags %u); results are invalid", v);
  }
  return NB_OK;
}

}  // namespace nb

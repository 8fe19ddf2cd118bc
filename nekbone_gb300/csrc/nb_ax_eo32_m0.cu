// Even-odd FP32 element operator instantiations, mode 0 (nb_kernels.cuh).
#include "nb_ax_eo_launch.cuh"

namespace nb {
int launch_ax_eo32_m0(int lx, AxArgs<float> a, const double *eo, cudaStream_t s) {
  return launch_ax_eo_mode<float, 0>(lx, a, eo, s);
}
}  // namespace nb

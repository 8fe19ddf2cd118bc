// Element operator instantiations: float, mode 1 (see nb_kernels.cuh).
#include "nb_ax_launch.cuh"

namespace nb {
int launch_ax_f32_m1(int lx, AxArgs<float> a, cudaStream_t s) {
  return launch_ax_mode<float, 1>(lx, a, s);
}
}  // namespace nb

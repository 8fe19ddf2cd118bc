// Element operator instantiations: float, mode 2 (see nb_kernels.cuh).
#include "nb_ax_launch.cuh"

namespace nb {
int launch_ax_f32_m2(int lx, AxArgs<float> a, cudaStream_t s) {
  return launch_ax_mode<float, 2>(lx, a, s);
}
}  // namespace nb

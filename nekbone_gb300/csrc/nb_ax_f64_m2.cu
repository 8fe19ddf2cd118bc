// Element operator instantiations: double, mode 2 (see nb_kernels.cuh).
#include "nb_ax_launch.cuh"

namespace nb {
int launch_ax_f64_m2(int lx, AxArgs<double> a, cudaStream_t s) {
  return launch_ax_mode<double, 2>(lx, a, s);
}
}  // namespace nb

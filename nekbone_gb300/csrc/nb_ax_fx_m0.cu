// nb_ax_fx_m0.cu -- fixed-point FP64 element operator, MODE 0.
#include "nb_ax_fx_launch.cuh"

namespace nb {
int launch_ax_fx_m0(const Operator &op, AxArgs<double> a, cudaStream_t s) {
  return launch_ax_fx_mode<0>(op, a, s);
}
}  // namespace nb

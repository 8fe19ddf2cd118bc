// nb_ax_fx_m1.cu -- fixed-point FP64 element operator, MODE 1.
#include "nb_ax_fx_launch.cuh"

namespace nb {
int launch_ax_fx_m1(const Operator &op, AxArgs<double> a, cudaStream_t s) {
  return launch_ax_fx_mode<1>(op, a, s);
}
}  // namespace nb

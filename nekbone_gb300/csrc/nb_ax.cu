// nb_ax.cu -- launch_ax<T>: the element operator for a mesh and mode.
#include "nb_solver.h"

namespace nb {

int launch_ax_f64_m0(int lx, AxArgs<double> a, cudaStream_t s);
int launch_ax_f64_m1(int lx, AxArgs<double> a, cudaStream_t s);
int launch_ax_f64_m2(int lx, AxArgs<double> a, cudaStream_t s);
int launch_ax_eo_m0(int lx, AxArgs<double> a, const double *eo, cudaStream_t s);
int launch_ax_eo_m1(int lx, AxArgs<double> a, const double *eo, cudaStream_t s);
int launch_ax_eo_m2(int lx, AxArgs<double> a, const double *eo, cudaStream_t s);
int launch_ax_eo32_m0(int lx, AxArgs<float> a, const double *eo, cudaStream_t s);
int launch_ax_eo32_m1(int lx, AxArgs<float> a, const double *eo, cudaStream_t s);
int launch_ax_f32_m0(int lx, AxArgs<float> a, cudaStream_t s);
int launch_ax_f32_m1(int lx, AxArgs<float> a, cudaStream_t s);
int launch_ax_f32_m2(int lx, AxArgs<float> a, cudaStream_t s);
int launch_ax_fx_m0(const Operator &op, AxArgs<double> a, cudaStream_t s);
int launch_ax_fx_m1(const Operator &op, AxArgs<double> a, cudaStream_t s);
int launch_ax_fx_m2(const Operator &op, AxArgs<double> a, cudaStream_t s);

template <>
int launch_ax<double>(const Operator &op, int mode, AxArgs<double> a, cudaStream_t s) {
  a.nelt = op.nelt;
  if (!a.pold) a.pold = a.p;  // MODE 1 reads the old direction from pold
  a.err = device_error_word();
  a.wait_test = wait_test_mode();
  if (op.order == 2 && op.fx_ok) {  // fixed point on the integer pipes
    NB_TRY(metric_fx_prepare(op, a.g, s));
    a.gfx = op.gfx;
    a.gexp = op.gexp;
    if (mode == 0) return launch_ax_fx_m0(op, a, s);
    if (mode == 1) return launch_ax_fx_m1(op, a, s);
    return launch_ax_fx_m2(op, a, s);
  }
  if (op.order >= 1 && op.eo_ok) {  // even-odd split (FP64 pipe bound)
    if (mode == 0) return launch_ax_eo_m0(op.lx, a, op.EO.data(), s);
    if (mode == 1) return launch_ax_eo_m1(op.lx, a, op.EO.data(), s);
    return launch_ax_eo_m2(op.lx, a, op.EO.data(), s);
  }
  if (mode == 0) return launch_ax_f64_m0(op.lx, a, s);
  if (mode == 1) return launch_ax_f64_m1(op.lx, a, s);
  return launch_ax_f64_m2(op.lx, a, s);
}

template <>
int launch_ax<float>(const Operator &op, int mode, AxArgs<float> a, cudaStream_t s) {
  a.nelt = op.nelt;
  if (!a.pold) a.pold = a.p;  // MODE 1 reads the old direction from pold
  a.err = device_error_word();
  a.wait_test = wait_test_mode();
  if (op.order >= 1 && op.eo_ok && mode != 2) {  // even-odd, one line per thread
    if (mode == 0) return launch_ax_eo32_m0(op.lx, a, op.EO.data(), s);
    return launch_ax_eo32_m1(op.lx, a, op.EO.data(), s);
  }
  if (mode == 0) return launch_ax_f32_m0(op.lx, a, s);
  if (mode == 1) return launch_ax_f32_m1(op.lx, a, s);
  return launch_ax_f32_m2(op.lx, a, s);
}

}  // namespace nb

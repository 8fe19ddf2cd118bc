// nb_ax_fx_launch.cuh -- dispatch of the fixed-point FP64 element operator
// over even lx1 (one translation unit per mode includes this).
#pragma once

#include "nb_ax_fx.cuh"
#include "nb_solver.h"

namespace nb {

template <int LX, int MODE>
int launch_ax_fx_shape(const Operator &op, AxArgs<double> a, cudaStream_t s) {
  const size_t sm = fx::ax_fx_smem_bytes<LX>();
  static bool attr_set = false;
  if (!attr_set) {
    NB_CUDA(cudaFuncSetAttribute(fx::k_ax_fx<LX, MODE>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
    attr_set = true;
  }
  constexpr int Q = 4 * (LX / 2) * (LX / 2);
  if (int(op.FXhi.size()) != Q || int(op.FXlo.size()) != Q)
    return fail(NB_ERR_STATE, "fixed-point ax: tables for lx1=%d missing", LX);
  fx::FxCoef<LX> cf;
  for (int q = 0; q < Q; ++q) {
    cf.hi[q] = op.FXhi[q];
    cf.lo[q] = op.FXlo[q];
  }
  cf.fc = op.fx_fc;
  fx::k_ax_fx<LX, MODE><<<a.nelt, dim3(LX, LX), sm, s>>>(a, cf);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

template <int MODE>
int launch_ax_fx_mode(const Operator &op, AxArgs<double> a, cudaStream_t s) {
  switch (op.lx) {
#define NB_CASE(L) case L: return launch_ax_fx_shape<L, MODE>(op, a, s);
    NB_CASE(2) NB_CASE(4) NB_CASE(6) NB_CASE(8) NB_CASE(10) NB_CASE(12) NB_CASE(14) NB_CASE(16)
#undef NB_CASE
    default:
      return fail(NB_ERR_UNSUPPORTED, "fixed-point ax: lx1=%d", op.lx);
  }
}

}  // namespace nb

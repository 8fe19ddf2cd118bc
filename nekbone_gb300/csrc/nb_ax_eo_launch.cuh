// nb_ax_eo_launch.cuh -- dispatch of the even-odd FP64 operator over even lx1.
#pragma once

#include "nb_solver.h"

namespace nb {

template <int LX, int MODE>
int launch_ax_eo_lx(AxArgs<double> a, const double *eo, cudaStream_t s) {
  const size_t sm = ax_eo_smem_bytes<LX>();
  static bool attr_set = false;
  if (!attr_set) {
    NB_CUDA(cudaFuncSetAttribute(k_ax_eo<LX, MODE>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
    attr_set = true;
  }
  k_ax_eo<LX, MODE><<<a.nelt, dim3(LX, LX), sm, s>>>(a, eo);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

template <int MODE>
int launch_ax_eo_mode(int lx, AxArgs<double> a, const double *eo, cudaStream_t s) {
  switch (lx) {
#define NB_CASE(L) case L: return launch_ax_eo_lx<L, MODE>(a, eo, s);
    NB_CASE(2) NB_CASE(4) NB_CASE(6) NB_CASE(8) NB_CASE(10) NB_CASE(12) NB_CASE(14) NB_CASE(16)
#undef NB_CASE
    default:
      return fail(NB_ERR_UNSUPPORTED, "even-odd ax: lx1=%d", lx);
  }
}

}  // namespace nb

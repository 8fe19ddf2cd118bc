// nb_ax_launch.cuh -- dispatch of the element operator over lx1 (2..16).
#pragma once

#include <type_traits>

#include "nb_solver.h"

namespace nb {

// FP32, even lx1, modes 0/1, metric pointer 16-byte aligned: the bulk-copy
// kernel; otherwise the general one.
template <int LX, int MODE>
int launch_ax_f32_tma(AxArgs<float> a, cudaStream_t s) {
  const size_t sm = ax_tma_smem_bytes<LX>();
  static bool attr_set = false;
  if (!attr_set) {
    NB_CUDA(cudaFuncSetAttribute(k_ax_f32_tma<LX, MODE>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
    attr_set = true;
  }
  k_ax_f32_tma<LX, MODE><<<a.nelt, dim3(LX, LX), sm, s>>>(a);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

template <typename T, int LX, int MODE>
int launch_ax_lx(AxArgs<T> a, cudaStream_t s) {
  constexpr bool RD = std::is_same<T, float>::value;
  if constexpr (std::is_same<T, float>::value && LX % 2 == 0 && MODE != 2 &&
                sizeof(AxTmaShared<LX>) <= 227 * 1024) {
    if ((reinterpret_cast<uintptr_t>(a.g) & 15u) == 0)
      return launch_ax_f32_tma<LX, MODE>(reinterpret_cast<AxArgs<float> &>(a), s);
  }
  const size_t sm = ax_smem_bytes<T, LX>();
  static bool attr_set = false;
  if (!attr_set) {
    NB_CUDA(cudaFuncSetAttribute(k_ax_impl<T, LX, MODE, RD>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
    attr_set = true;
  }
  k_ax_impl<T, LX, MODE, RD><<<a.nelt, dim3(LX, LX), sm, s>>>(a);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

template <typename T, int MODE>
int launch_ax_mode(int lx, AxArgs<T> a, cudaStream_t s) {
  switch (lx) {
#define NB_CASE(L) case L: return launch_ax_lx<T, L, MODE>(a, s);
    NB_CASE(2) NB_CASE(3) NB_CASE(4) NB_CASE(5) NB_CASE(6) NB_CASE(7)
    NB_CASE(8) NB_CASE(9) NB_CASE(10) NB_CASE(11) NB_CASE(12) NB_CASE(13)
    NB_CASE(14) NB_CASE(15) NB_CASE(16)
#undef NB_CASE
    default:
      return fail(NB_ERR_UNSUPPORTED, "ax: lx1=%d not supported (2..%d)", lx, kMaxLx);
  }
}

}  // namespace nb

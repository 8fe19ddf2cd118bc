// nb_ax_eo_launch.cuh -- dispatch of the even-odd element operator (FP64 and
// FP32) over even lx1.
#pragma once

#include "nb_solver.h"

namespace nb {

// eo: the even-odd tables on the host (FP64); each launch carries them,
// rounded to T, as its EoCoef parameter.
template <typename T, int LX, int MODE, bool TMAG>
int launch_ax_eo_shape(AxArgs<T> a, const double *eo, cudaStream_t s) {
  const size_t sm = ax_eo_smem_bytes<T, LX, TMAG>();
  // FP64 at lx1 = 12 (CG and apply): the four-CTA form, 96 registers with
  // a few bytes spilled, keeps four CTAs per SM instead of two at 134
  // registers (FP64 pipe 92 % busy instead of 86 %); the other shapes spill
  // too much under that cap
  void (*fn)(AxArgs<T>, const EoCoef<T, LX>);
  if constexpr (sizeof(T) == 8 && LX == 12 && MODE != 2) fn = k_ax_eo4<T, LX, MODE, TMAG>;
  else fn = k_ax_eo<T, LX, MODE, TMAG>;
  static bool attr_set = false;
  if (!attr_set) {
    NB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
    attr_set = true;
  }
  EoCoef<T, LX> cf;
  eo_fill(cf, eo);
  fn<<<a.nelt, dim3(LX, LX), sm, s>>>(a, cf);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

// FP32 with a 16-byte aligned per-element metric: the bulk-copy (TMAG)
// form.  A shared metric block (g_uniform) is read directly: it stays
// cache-resident, and without the copy's shared memory more CTAs fit.
template <typename T, int LX, int MODE>
int launch_ax_eo_lx(AxArgs<T> a, const double *eo, cudaStream_t s) {
  if constexpr (sizeof(T) == 4 && MODE != 2 && (24 * LX * LX * LX) % 16 == 0) {
    if (!a.g_uniform && (reinterpret_cast<uintptr_t>(a.g) & 15u) == 0)
      return launch_ax_eo_shape<T, LX, MODE, true>(a, eo, s);
  }
  return launch_ax_eo_shape<T, LX, MODE, false>(a, eo, s);
}

template <typename T, int MODE>
int launch_ax_eo_mode(int lx, AxArgs<T> a, const double *eo, cudaStream_t s) {
  switch (lx) {
#define NB_CASE(L) case L: return launch_ax_eo_lx<T, L, MODE>(a, eo, s);
    NB_CASE(2) NB_CASE(4) NB_CASE(6) NB_CASE(8) NB_CASE(10) NB_CASE(12) NB_CASE(14) NB_CASE(16)
#undef NB_CASE
    default:
      return fail(NB_ERR_UNSUPPORTED, "even-odd ax: lx1=%d", lx);
  }
}

}  // namespace nb

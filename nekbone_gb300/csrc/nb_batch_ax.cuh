// nb_batch_ax.cuh -- the element operator of many problems at once.
//
// A CTA holds EPB elements of one lx1 (thread tile lx1 x lx1 x EPB; thread
// (i,j,z) owns column (i,j,.) of element z), which may belong to different
// problems: every element looks up its own problem's scalars (beta, or the
// defect scale |r|) and skips all work when its problem has converged.  The
// contractions are those of the single-mesh operator (local_grad3 /
// local_grad3_t, cg.f:170-212, in the mxfN left-to-right order); RD selects
// D in registers with vector shared-memory loads (the FP32 form) or padded
// shared D (the FP64 form).  Element partials of the CG dot products are
// reduced in a fixed order (rows, then the element) into partial[e].
#pragma once

#include "nb_batch.h"

namespace nb {

template <typename T, int LX, int EPB>
struct BaxShared {
  struct Elem {
    alignas(16) T u[LX * LX * LX];
    alignas(16) T wr[LX * LX * LX];
    alignas(16) T ws[LX * LX * LX];
  } el[EPB];
  T Dp[LX * (LX + 1)];   // Dp[i*(LX+1)+m] = D(i,m)
  T Dtp[LX * (LX + 1)];  // Dtp[i*(LX+1)+m] = D(m,i)
  alignas(16) T Dr[LX * LX];  // Dr[k*LX+m] = D(k,m)
  alignas(16) T Dc[LX * LX];  // Dc[k*LX+m] = D(m,k)
  T part[EPB][LX * LX];
  double row[EPB][LX];
};

template <typename T, int LX, int MODE, bool RD, int EPB>
__global__ void __launch_bounds__(LX * LX * EPB)
    k_bax(BaxArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  BaxShared<T, LX, EPB> &sm = *reinterpret_cast<BaxShared<T, LX, EPB> *>(smem_raw);
  constexpr int L2 = LX * LX, L3 = LX * LX * LX, LP = LX + 1;
  const int i = threadIdx.x, j = threadIdx.y, z = threadIdx.z;
  const int tid = i + LX * j;
  const int tflat = tid + L2 * z;
  const int el = blockIdx.x * EPB + z;
  const bool in_range = el < a.nel;
  const int e = a.el0 + (in_range ? el : 0);
  const int prob = a.el_prob[e];
  // the inner operator (MODE 1) skips problems whose inner CG ended
  const bool act = in_range && a.sc[prob].active && (MODE != 1 || a.sc[prob].iactive);
  if (!__syncthreads_or(act)) return;  // every element of the CTA converged
  const size_t base = size_t(a.pt0) + size_t(in_range ? el : 0) * L3;
  auto &E = sm.el[z];

  if (tflat < L2) {
    const int r = tflat % LX, m = tflat / LX;  // D(r,m)
    const T d = a.D[r + m * LX];
    if (RD) {
      sm.Dr[r * LX + m] = d;
      sm.Dc[m * LX + r] = d;
    } else {
      sm.Dp[r * LP + m] = d;
      sm.Dtp[m * LP + r] = d;
    }
  }

  T ureg[LX];
  const bool col_interior = (i > 0) && (i < LX - 1) && (j > 0) && (j < LX - 1);
  T creg[LX], freg[LX];
  T beta = T(0);
  T scale = T(0);
  if (act) {
    if (MODE == 1 && !a.first) beta = T(a.sc[prob].beta);
    if (MODE == 2) scale = T(a.sc[prob].rn);
    if (col_interior) {
#pragma unroll
      for (int k = 1; k < LX - 1; ++k) {
        const size_t id = base + size_t(k) * L2 + tid;
        creg[k] = (MODE == 1 && a.c_unit_interior) ? T(1) : a.c[id];
        if (MODE == 2) freg[k] = a.f[id];
      }
    }
  }
  T pold[LX];
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + tid;
    ureg[k] = T(0);
    pold[k] = T(0);
    if (act) {
      if (MODE == 1) {
        ureg[k] = a.u[id];
        if (!a.first) pold[k] = a.pold[id];
      } else {
        ureg[k] = a.p[id];
        pold[k] = T(a.e[id]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + tid;
    if (MODE == 1) {
      if (!a.first) ureg[k] = fma_rn(beta, pold[k], ureg[k]);  // add2s1, math.f:534
      if (act) a.p[id] = ureg[k];
    } else {
      ureg[k] = fma_rn(scale, pold[k], ureg[k]);  // x += |r| e
      if (act) a.p[id] = ureg[k];
    }
    E.u[k * L2 + tid] = ureg[k];
  }
  __syncthreads();

  T Di[RD ? LX : 1], Dj[RD ? LX : 1];
  if (RD) {
#pragma unroll
    for (int m = 0; m < LX; ++m) {
      Di[m] = sm.Dr[i * LX + m];
      Dj[m] = sm.Dr[j * LX + m];
    }
  }

  T wtreg[LX];
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    T ur, us, ut;
    const T *urow = &E.u[k * L2 + j * LX];
    const T *ucol = &E.u[k * L2 + i];
    if (RD) {
      ur = dot_contig<T, LX>(Di, urow);
      us = mul_rn(ucol[0], Dj[0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) us = fma_rn(ucol[m * LX], Dj[m], us);
      ut = dot_contig<T, LX>(ureg, &sm.Dr[k * LX]);
    } else {
      ur = mul_rn(sm.Dp[i * LP + 0], urow[0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) ur = fma_rn(sm.Dp[i * LP + m], urow[m], ur);
      us = mul_rn(ucol[0], sm.Dp[j * LP + 0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) us = fma_rn(ucol[m * LX], sm.Dp[j * LP + m], us);
      ut = mul_rn(ureg[0], sm.Dp[k * LP + 0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) ut = fma_rn(ureg[m], sm.Dp[k * LP + m], ut);
    }
    T wr = T(0), ws = T(0), wt = T(0);
    if (act) {
      const size_t pt = base + size_t(k) * L2 + tid;
      typedef typename Vec2<T>::type V2;
      const V2 *gp = reinterpret_cast<const V2 *>(a.g + 6 * pt);
      const V2 g01 = gp[0], g23 = gp[1], g45 = gp[2];
      wr = mul_rn(g01.x, ur);
      wr = fma_rn(g01.y, us, wr);
      wr = fma_rn(g23.x, ut, wr);
      ws = mul_rn(g01.y, ur);
      ws = fma_rn(g23.y, us, ws);
      ws = fma_rn(g45.x, ut, ws);
      wt = mul_rn(g23.x, ur);
      wt = fma_rn(g45.x, us, wt);
      wt = fma_rn(g45.y, ut, wt);
    }
    E.wr[k * L2 + tid] = wr;
    E.ws[k * L2 + tid] = ws;
    wtreg[k] = wt;
  }
  __syncthreads();

  if (RD) {
#pragma unroll
    for (int m = 0; m < LX; ++m) {
      Di[m] = sm.Dc[i * LX + m];
      Dj[m] = sm.Dc[j * LX + m];
    }
  }

  T part = T(0);
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    T tr, ts, tt;
    const T *rrow = &E.wr[k * L2 + j * LX];
    const T *scol = &E.ws[k * L2 + i];
    if (RD) {
      tr = dot_contig<T, LX>(Di, rrow);
      ts = mul_rn(scol[0], Dj[0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) ts = fma_rn(scol[m * LX], Dj[m], ts);
      tt = dot_contig<T, LX>(wtreg, &sm.Dc[k * LX]);
    } else {
      tr = mul_rn(sm.Dtp[i * LP + 0], rrow[0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) tr = fma_rn(sm.Dtp[i * LP + m], rrow[m], tr);
      ts = mul_rn(scol[0], sm.Dtp[j * LP + 0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) ts = fma_rn(scol[m * LX], sm.Dtp[j * LP + m], ts);
      tt = mul_rn(wtreg[0], sm.Dtp[k * LP + 0]);
#pragma unroll
      for (int m = 1; m < LX; ++m) tt = fma_rn(wtreg[m], sm.Dtp[k * LP + m], tt);
    }
    T wl = add_rn(add_rn(tr, ts), tt);
    const size_t id = base + size_t(k) * L2 + tid;
    const bool interior = col_interior && (k > 0) && (k < LX - 1);
    if (act) {
      if (MODE == 1) {
        if (interior) {
          wl = fma_rn(T(0.1), ureg[k], wl);  // add2s2(w,u,.1,n), cg.f:119
          part = fma_rn(mul_rn(wl, creg[k]), ureg[k], part);
        }
        a.w[id] = wl;
      } else {
        if (interior) {
          const T rv = freg[k] - fma_rn(T(0.1), ureg[k], wl);
          a.r[id] = rv;
          part = fma_rn(mul_rn(rv, creg[k]), rv, part);
        } else {
          a.w[id] = wl;
        }
      }
    }
  }
  // element partial: rows (i summed by thread (j,0)), then rows in order
  sm.part[z][tid] = part;
  __syncthreads();
  if (tid < LX) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < LX; ++q) s += double(sm.part[z][q + LX * tid]);
    sm.row[z][tid] = s;
  }
  __syncthreads();
  if (tid == 0 && act) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < LX; ++q) s += sm.row[z][q];
    a.partial[e] = s;
  }
}

// The even-odd form for the batch: one element per CTA, one 1-D line per
// thread in each contraction (the single-mesh k_ax_eo), with the per-element
// problem lookups of k_bax.  TMAG: the element's metric block arrives by one
// bulk copy (FP32).
template <typename T, int LX, int MODE, bool TMAG>
__global__ void __launch_bounds__(LX * LX)
    k_bax_eo(BaxArgs<T> a, const __grid_constant__ EoCoef<T, LX> cf) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AxEoShared<T, LX, TMAG> &sm = *reinterpret_cast<AxEoShared<T, LX, TMAG> *>(smem_raw);
  constexpr int L2 = LX * LX, L3 = LX * LX * LX, H = LX / 2;
  const int t = threadIdx.x + LX * threadIdx.y;
  const int i = threadIdx.x, j = threadIdx.y;
  const int e = a.el0 + blockIdx.x;
  const int prob = a.el_prob[e];
  if (!a.sc[prob].active || (MODE == 1 && !a.sc[prob].iactive)) return;  // one element
  const size_t base = size_t(a.pt0) + size_t(blockIdx.x) * L3;
  if (TMAG && t == 0)
    block_copy_begin(&sm.bar, sm.g, a.g + 6 * base, unsigned(6 * L3 * sizeof(T)), a.wait_test);
  // coefficients as in k_ax_eo: FP32 from the parameter bank, FP64 staged
  // in shared memory
  constexpr bool CPAR = sizeof(T) == 4 && LX <= 12;
  if constexpr (!CPAR)
    for (int q = t; q < 4 * H * H; q += L2) sm.E4[q] = cf.c[q];
  const T *E4 = CPAR ? cf.c : sm.E4;
  const T *Ed = E4, *Od = E4 + H * H;
  const T *Et = E4 + 2 * H * H, *Ot = E4 + 3 * H * H;

  constexpr bool DEALT = eo_dealt<T, LX>();
  const int lr = DEALT ? int(cf.rmap[t]) : t, ls = DEALT ? int(cf.smap[t]) : t;
  const int r0 = lr % LX, r1 = lr / LX, s0 = ls % LX, s1 = ls / LX;

  const bool col_interior = (i > 0) && (i < LX - 1) && (j > 0) && (j < LX - 1);
  T creg[LX], freg[LX];
  if (col_interior) {
#pragma unroll
    for (int k = 1; k < LX - 1; ++k) {
      const size_t id = base + size_t(k) * L2 + t;
      creg[k] = (MODE == 1 && a.c_unit_interior) ? T(1) : a.c[id];
      if (MODE == 2) freg[k] = a.f[id];
    }
  }
  T ureg[LX], pold[LX];
  const T beta = (MODE == 1 && !a.first) ? T(a.sc[prob].beta) : T(0);
  const T scale = MODE == 2 ? T(a.sc[prob].rn) : T(0);
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + t;
    if (MODE == 1) {
      ureg[k] = a.u[id];
      pold[k] = a.first ? T(0) : a.pold[id];
    } else {
      ureg[k] = a.p[id];
      pold[k] = T(a.e[id]);
    }
  }
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + t;
    if (MODE == 1) {
      if (!a.first) ureg[k] = fma_rn(beta, pold[k], ureg[k]);
    } else {
      ureg[k] = fma_rn(scale, pold[k], ureg[k]);
    }
    a.p[id] = ureg[k];
    sm.A[eo_at<T, LX>(i, j, k)] = ureg[k];
  }
  __syncthreads();
  {
    T v[LX], y[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.A[eo_at<T, LX>(m, r0, r1)];
    eo_line<T, LX>(v, Ed, Od, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.B[eo_at<T, LX>(m, r0, r1)] = y[m];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.A[eo_at<T, LX>(s0, m, s1)];
    eo_line<T, LX>(v, Ed, Od, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.C[eo_at<T, LX>(s0, m, s1)] = y[m];
  }
  T wtreg[LX];
  eo_line<T, LX>(ureg, Ed, Od, wtreg);
  __syncthreads();
  if (TMAG && !block_copy_wait(&sm.bar, a.err, a.wait_test, sm.red, a.g + 6 * base)) return;
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const int q = eo_at<T, LX>(i, j, k);
    const T ur = sm.B[q], us = sm.C[q], ut = wtreg[k];
    const size_t pt = base + size_t(k) * L2 + t;
    typedef typename Vec2<T>::type V2;
    const V2 *gp = TMAG ? reinterpret_cast<const V2 *>(&sm.g[6 * (k * L2 + t)])
                        : reinterpret_cast<const V2 *>(a.g + 6 * pt);
    const V2 g01 = gp[0], g23 = gp[1], g45 = gp[2];
    T wr = mul_rn(g01.x, ur);
    wr = fma_rn(g01.y, us, wr);
    wr = fma_rn(g23.x, ut, wr);
    T ws = mul_rn(g01.y, ur);
    ws = fma_rn(g23.y, us, ws);
    ws = fma_rn(g45.x, ut, ws);
    T wt = mul_rn(g23.x, ur);
    wt = fma_rn(g45.x, us, wt);
    wt = fma_rn(g45.y, ut, wt);
    sm.B[q] = wr;
    sm.C[q] = ws;
    wtreg[k] = wt;
  }
  __syncthreads();
  {
    T v[LX], y[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.B[eo_at<T, LX>(m, r0, r1)];
    eo_line<T, LX>(v, Et, Ot, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.A[eo_at<T, LX>(m, r0, r1)] = y[m];
  }
  __syncthreads();
  {
    T v[LX], y[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.C[eo_at<T, LX>(s0, m, s1)];
    eo_line<T, LX>(v, Et, Ot, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.B[eo_at<T, LX>(s0, m, s1)] = y[m];
  }
  T ttreg[LX];
  eo_line<T, LX>(wtreg, Et, Ot, ttreg);
  __syncthreads();
  T part = T(0);
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const int q = eo_at<T, LX>(i, j, k);
    T wl = add_rn(add_rn(sm.A[q], sm.B[q]), ttreg[k]);
    const size_t id = base + size_t(k) * L2 + t;
    const bool interior = col_interior && (k > 0) && (k < LX - 1);
    if (MODE == 1) {
      if (interior) {
        wl = fma_rn(T(0.1), ureg[k], wl);
        part = fma_rn(mul_rn(wl, creg[k]), ureg[k], part);
      }
      a.w[id] = wl;
    } else {
      if (interior) {
        const T rv = freg[k] - fma_rn(T(0.1), ureg[k], wl);
        a.r[id] = rv;
        part = fma_rn(mul_rn(rv, creg[k]), rv, part);
      } else {
        a.w[id] = wl;
      }
    }
  }
  const double s = block_sum<T>(part, sm.red);
  if (t == 0) a.partial[e] = s;
}

template <typename T, int LX, int MODE>
int launch_bax_eo(const BaxArgs<T> &a, cudaStream_t s) {
  if constexpr (LX % 2 != 0) {
    return fail(NB_ERR_UNSUPPORTED, "batched even-odd operator: odd lx1=%d", LX);
  } else {
    constexpr bool TMAG = sizeof(T) == 4;   // element metric blocks are 16-byte aligned
    const size_t smem = sizeof(AxEoShared<T, LX, TMAG>);
    static bool attr = false;
    if (!attr) {
      NB_CUDA(cudaFuncSetAttribute(k_bax_eo<T, LX, MODE, TMAG>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
      attr = true;
    }
    if (a.nel <= 0) return NB_OK;
    if (!a.eo_h) return fail(NB_ERR_STATE, "batched even-odd operator: no tables");
    if (TMAG && (reinterpret_cast<uintptr_t>(a.g + 6 * a.pt0) & 15u))
      return fail(NB_ERR_STATE, "batched even-odd operator: metric not 16-byte aligned");
    EoCoef<T, LX> cf;
    eo_fill(cf, a.eo_h);
    k_bax_eo<T, LX, MODE, TMAG><<<a.nel, dim3(LX, LX), smem, s>>>(a, cf);
    NB_CUDA(cudaGetLastError());
    return NB_OK;
  }
}

template <typename T, int LX, int MODE, bool RD, int EPB>
int launch_bax(const BaxArgs<T> &a, cudaStream_t s) {
  const size_t smem = sizeof(BaxShared<T, LX, EPB>);
  static bool attr = false;
  if (!attr) {
    NB_CUDA(cudaFuncSetAttribute(k_bax<T, LX, MODE, RD, EPB>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    attr = true;
  }
  const int grid = (a.nel + EPB - 1) / EPB;
  if (grid <= 0) return NB_OK;
  k_bax<T, LX, MODE, RD, EPB><<<grid, dim3(LX, LX, EPB), smem, s>>>(a);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

// The shapes instantiated for lx1 = LX: three element counts per block
// (chosen so the thread tile stays within 64..576 threads), both D forms
// for FP32, and two counts for FP64.
template <int LX> struct BaxEpb;
template <> struct BaxEpb<4> { static constexpr int a = 4, b = 8, c = 16; };
template <> struct BaxEpb<6> { static constexpr int a = 2, b = 4, c = 8; };
template <> struct BaxEpb<8> { static constexpr int a = 1, b = 2, c = 4; };
template <> struct BaxEpb<10> { static constexpr int a = 1, b = 2, c = 4; };
template <> struct BaxEpb<12> { static constexpr int a = 1, b = 2, c = 4; };

template <int LX>
int batch_ax_f32_lx(int epb, int rd, const BaxArgs<float> &a, cudaStream_t s) {
  typedef BaxEpb<LX> P;
  if (rd == 2) {
    if (epb == 1) return launch_bax_eo<float, LX, 1>(a, s);
  } else if (rd) {
    if (epb == P::a) return launch_bax<float, LX, 1, true, P::a>(a, s);
    if (epb == P::b) return launch_bax<float, LX, 1, true, P::b>(a, s);
    if (epb == P::c) return launch_bax<float, LX, 1, true, P::c>(a, s);
  } else {
    if (epb == P::a) return launch_bax<float, LX, 1, false, P::a>(a, s);
    if (epb == P::b) return launch_bax<float, LX, 1, false, P::b>(a, s);
    if (epb == P::c) return launch_bax<float, LX, 1, false, P::c>(a, s);
  }
  return fail(NB_ERR_UNSUPPORTED, "batched FP32 operator: no shape epb=%d rd=%d for lx1=%d",
              epb, rd, LX);
}

template <int LX>
int batch_ax_f64_lx(int epb, const BaxArgs<double> &a, cudaStream_t s) {
  typedef BaxEpb<LX> P;
  if (epb == 0) return launch_bax_eo<double, LX, 2>(a, s);   // even-odd form
  if (epb == P::a) return launch_bax<double, LX, 2, false, P::a>(a, s);
  if (epb == P::b) return launch_bax<double, LX, 2, false, P::b>(a, s);
  return fail(NB_ERR_UNSUPPORTED, "batched FP64 operator: no shape epb=%d for lx1=%d", epb, LX);
}

#define NB_BATCH_AX_INSTANTIATE(LX)                                                       \
  template int batch_ax_f32_lx<LX>(int, int, const BaxArgs<float> &, cudaStream_t); \
  template int batch_ax_f64_lx<LX>(int, const BaxArgs<double> &, cudaStream_t);

}  // namespace nb

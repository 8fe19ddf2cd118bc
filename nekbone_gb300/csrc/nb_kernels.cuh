// nb_kernels.cuh -- device kernels of the Nekbone CG hot path.
//
// ax_e (cg.f:142-168) is evaluated one element per CTA with an (lx1 x lx1)
// thread tile: thread (i,j) owns the column (i,j,0..lx1-1).  The element is
// staged in shared memory; the t-direction contractions use the thread's own
// column held in registers.  Every contraction is the reference's
// left-to-right sum (mxfN, mxm_std.f:255) written as an explicit product
// followed by a fused multiply-add chain, so the FP64 result equals the
// oracle's fma variant bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace nb {

// ----------------------------------------------------------- arithmetic --
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

template <typename T> struct Vec2;
template <> struct Vec2<double> { typedef double2 type; };
template <> struct Vec2<float> { typedef float2 type; };

// counter-based uniform [-1,1) keyed by (seed, global id): splitmix64 finaliser
__device__ __forceinline__ double uniform_pm1(uint64_t seed, uint64_t id) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + id + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return double(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// ------------------------------------------------------------ reduction --
// Deterministic block sum of one value per thread: a fixed shuffle tree in
// the accumulation type A (float for the FP32 kernels, which keeps FP64
// instructions off the per-point path), then the per-warp results summed in
// FP64 in a fixed order.  Result valid in thread 0.
template <typename A>
__device__ __forceinline__ double block_sum(A v, double *sh) {
  const int lane = threadIdx.x + threadIdx.y * blockDim.x;
  const int nt = blockDim.x * blockDim.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = lane >> 5, nw = (nt + 31) >> 5;
  __syncthreads();
  if ((lane & 31) == 0) sh[w] = double(v);
  __syncthreads();
  double s = 0.0;
  if (lane == 0)
    for (int q = 0; q < nw; ++q) s += sh[q];
  return s;
}

// Sum of partial[0..n) in a fixed order by one block (result in thread 0).
__device__ __forceinline__ double block_sum_array(const double *partial, int n,
                                                  double *sh) {
  const int t = threadIdx.x + threadIdx.y * blockDim.x;
  const int nt = blockDim.x * blockDim.y;
  double v = 0.0;
  for (int q = t; q < n; q += nt) v += partial[q];
  return block_sum<double>(v, sh);
}

// Returns true in the block that finished last (all threads), after its
// partial is visible.  counter is reset for the next launch.
__device__ __forceinline__ bool last_block(unsigned *counter, int nblocks) {
  __shared__ bool amlast;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const unsigned prev = atomicAdd(counter, 1u);
    amlast = (prev == unsigned(nblocks) - 1u);
    if (amlast) *counter = 0u;
  }
  __syncthreads();
  if (amlast) __threadfence();
  return amlast;
}

// CG scalars, device resident (cg.f:27-75 variables).
struct CgScalars {
  double rtz1, rtz2, beta, pap, alpha, rtr, rnorm;
  double rtr_first;  // rtr of iteration 1 (cg.f:68)
  double alpha_prev;  // alpha of the iteration whose x update was deferred
  int iter;
  int pad;
};

// ------------------------------------------------------------ ax kernel --
// MODE 0: w = A_L u for every point (the element loop of ax, cg.f:111-114).
// MODE 1: fused CG pass -- p = z + beta*p (p = z when first), stored; the
//         element product w_L = A_L p; interior points (not shared, never
//         masked) are finished here: w = w_L + 0.1 p (ax, cg.f:119); element
//         boundary points keep w_L for the gather-scatter pass; the interior
//         part of pap = glsc3(w,c,p) goes to partial[blockIdx.x].
// MODE 2: fused defect pass of the mixed solver -- x += scale*e (when e is
//         given), w_L = A_L x; interior points get r = f - (w_L + 0.1 x) and
//         the interior part of r'Cr; boundary points keep w_L.
template <typename T>
struct AxArgs {
  T *w;
  const T *u;        // MODE 0 input; MODE 1: z
  T *p;              // MODE 1: search direction (read old, write new); MODE 2: x
  const T *pold;     // MODE 1: the old direction, read from here (another
                     //   buffer than p when the directions alternate; launch_ax
                     //   sets it to p when null: a select of the two pointers
                     //   in the kernel measured 25 % slower, FP32 at 32^3)
  const T *g;        // gxyz(6, nxyz, nelt)
  const T *c;        // MODE 1/2: inverse multiplicity
  const T *D;        // dxm1(lx1,lx1) column-major: D(i,m) at D[i + m*lx1]
  const CgScalars *sc;
  double *partial;
  int first;         // MODE 1: first iteration (beta = 0)
  int nelt;
  const T *f;        // MODE 2: right-hand side
  T *r;              // MODE 2: residual (interior points)
  const float *e;    // MODE 2: FP32 correction added to x first (may be null)
  double scale;      // MODE 2: its scale
  unsigned *err;     // device error word for bounded waits (may be null)
  int g_uniform;     // every element's metric block equals element 0's: read that one
  int wait_test;     // timeout self-test of the bulk-copy wait (block_copy_begin)
  const int2 *gfx;   // fixed-point FP64 operator: the metric in fixed point
  const int *gexp;   //   and each element's exponent (metric_fx_prepare)
  const int *el_prob;  // fixed-point operator in a batched solve: element e is
  const int *act;      //   skipped when act[el_prob[e] * act_stride] is 0 (its
  int act_stride;      //   problem is no longer active); null for one mesh
  int c_unit_interior;  // MODE 1: c is 1 at every element-interior point (a
                        //   verified multiplicity): not read there
};

template <typename T, int LX>
struct AxShared {
  alignas(16) T u[LX * LX * LX];
  alignas(16) T wr[LX * LX * LX];
  alignas(16) T ws[LX * LX * LX];
  T Dp[LX * (LX + 1)];   // Dp[i*(LX+1)+m] = D(i,m)   (FP64 kernel)
  T Dtp[LX * (LX + 1)];  // Dtp[i*(LX+1)+m] = D(m,i)  (FP64 kernel)
  alignas(16) T Dr[LX * LX];  // Dr[k*LX+m] = D(k,m)   (register-D kernel)
  alignas(16) T Dc[LX * LX];  // Dc[k*LX+m] = D(m,k)
  double red[32];
};

// Sum over m of coef[m] * data[m] in the reference's order (first product,
// then fused multiply-adds); data contiguous in shared memory and read with
// the widest aligned vector loads.
template <typename T, int LX>
__device__ __forceinline__ T dot_contig(const T *coef, const T *data) {
  T v[LX];
  if (sizeof(T) == 4 && LX % 4 == 0) {
#pragma unroll
    for (int q = 0; q < LX / 4; ++q) {
      const float4 t = reinterpret_cast<const float4 *>(data)[q];
      v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
    }
  } else if (sizeof(T) == 4 && LX % 2 == 0) {
#pragma unroll
    for (int q = 0; q < LX / 2; ++q) {
      const float2 t = reinterpret_cast<const float2 *>(data)[q];
      v[2 * q] = t.x; v[2 * q + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int q = 0; q < LX; ++q) v[q] = data[q];
  }
  T s = mul_rn(coef[0], v[0]);
#pragma unroll
  for (int m = 1; m < LX; ++m) s = fma_rn(coef[m], v[m], s);
  return s;
}

// Element operator.  RD (register D): the thread keeps D(i,:), D(j,:),
// D(:,i), D(:,j) in registers and reads rows of the element and of D with
// vector loads -- the FP32 variant, where shared-memory bandwidth, not
// arithmetic, limits; the FP64 variant reads D from padded shared memory
// (the FP64 pipe limits there, and registers go to occupancy).
template <typename T, int LX, int MODE, bool RD>
__global__ void __launch_bounds__(LX * LX)
    k_ax_impl(AxArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AxShared<T, LX> &sm = *reinterpret_cast<AxShared<T, LX> *>(smem_raw);
  constexpr int L2 = LX * LX, L3 = LX * LX * LX, LP = LX + 1;
  const int i = threadIdx.x, j = threadIdx.y;
  const int tid = i + LX * j;
  const int e = blockIdx.x;
  const size_t base = size_t(e) * L3;

  {
    const int r = tid % LX, m = tid / LX;  // D(r,m)
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
  // c (and f) are needed only at interior points; they are fetched with the
  // element, not inside the epilogue, so that no load waits behind a store
  const bool col_interior = (i > 0) && (i < LX - 1) && (j > 0) && (j < LX - 1);
  T creg[LX], freg[LX];
  if (MODE != 0 && col_interior) {
#pragma unroll
    for (int k = 1; k < LX - 1; ++k) {
      const size_t id = base + size_t(k) * L2 + tid;
      creg[k] = (MODE == 1 && a.c_unit_interior) ? T(1) : a.c[id];
      if (MODE == 2) freg[k] = a.f[id];
    }
  }
  T beta = T(0);
  if (MODE == 1 && !a.first) beta = T(a.sc->beta);
  // every load of the element is issued before the first store (p or x may
  // alias nothing, but the compiler cannot know: a store between loads would
  // serialise them)
  T pold[LX];
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + tid;
    if (MODE == 1) {
      ureg[k] = a.u[id];
      pold[k] = a.first ? T(0) : a.pold[id];
    } else if (MODE == 2) {
      ureg[k] = a.p[id];
      pold[k] = a.e ? T(a.e[id]) : T(0);
    } else {
      ureg[k] = a.u[id];
    }
  }
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + tid;
    if (MODE == 1) {
      if (!a.first) ureg[k] = fma_rn(beta, pold[k], ureg[k]);  // add2s1, math.f:534
      a.p[id] = ureg[k];
    } else if (MODE == 2 && a.e) {
      ureg[k] = fma_rn(T(a.scale), pold[k], ureg[k]);
      a.p[id] = ureg[k];
    }
    sm.u[k * L2 + tid] = ureg[k];
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
    // local_grad3, cg.f:170-187
    T ur, us, ut;
    const T *urow = &sm.u[k * L2 + j * LX];
    const T *ucol = &sm.u[k * L2 + i];
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
    // metric, cg.f:156-163
    const size_t pt = base + size_t(k) * L2 + tid;
    typedef typename Vec2<T>::type V2;
    const V2 *gp = reinterpret_cast<const V2 *>(a.g + 6 * pt);
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
    sm.wr[k * L2 + tid] = wr;
    sm.ws[k * L2 + tid] = ws;
    wtreg[k] = wt;
  }
  __syncthreads();

  if (RD) {
#pragma unroll
    for (int m = 0; m < LX; ++m) {
      Di[m] = sm.Dc[i * LX + m];  // D(m,i)
      Dj[m] = sm.Dc[j * LX + m];  // D(m,j)
    }
  }

  T part = T(0);
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    // local_grad3_t, cg.f:189-212: u = Dt*ur; w = us*D; u += w; w = ut*D; u += w
    T tr, ts, tt;
    const T *rrow = &sm.wr[k * L2 + j * LX];
    const T *scol = &sm.ws[k * L2 + i];
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
    if (MODE == 1) {
      if (interior) {
        wl = fma_rn(T(0.1), ureg[k], wl);  // add2s2(w,u,.1,n), cg.f:119
        part = fma_rn(mul_rn(wl, creg[k]), ureg[k], part);
      }
      a.w[id] = wl;
    } else if (MODE == 2) {
      if (interior) {
        const T rv = freg[k] - fma_rn(T(0.1), ureg[k], wl);
        a.r[id] = rv;
        part = fma_rn(mul_rn(rv, creg[k]), rv, part);
      } else {
        a.w[id] = wl;
      }
    } else {
      a.w[id] = wl;
    }
  }
  if (MODE != 0) {
    const double s = block_sum<T>(part, sm.red);
    if (i == 0 && j == 0) a.partial[e] = s;
  }
}

template <typename T, int LX>
constexpr size_t ax_smem_bytes() {
  return sizeof(AxShared<T, LX>);
}

// ------------------------------------------------ gather-scatter finish --
// For every group of element-boundary points: t = sum of w_L over the group
// in jl's member order (gather_T_add, jl/gs_local.c:60-75); each member gets
// w = t + 0.1 p (cg.f:119) or 0 when masked (maskit, cg.f:214-258); the
// boundary part of pap = glsc3(w,c,p) is reduced; the block that finishes
// last adds the interior partials, forms pap and alpha = rtz1/pap (cg.f:59-61).
// idx: member index in bits 0..30, mask flag in bit 31.
// four resident blocks per SM (64 registers; with more registers and two
// blocks the pass measured 0.56 ms instead of 0.40 ms, FP64 at 32^3), and
// the launch grid is exactly the resident blocks (nb_solver.cu)
#ifndef NB_GS_MINB
#define NB_GS_MINB 4
#endif
template <typename T>
__global__ void __launch_bounds__(256, NB_GS_MINB)
    k_gs_fin(T *__restrict__ w, const T *__restrict__ p,
             const T *__restrict__ c, const int *__restrict__ off,
             const unsigned *__restrict__ idx, int ng,
             double *__restrict__ partial, const double *__restrict__ ax_partial,
             int n_ax_partial, unsigned *counter, CgScalars *sc) {
  __shared__ double red[32];
  T part = T(0);
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng;
       g += gridDim.x * blockDim.x) {
    const int b = off[g], e = off[g + 1];
    T t = w[idx[b] & 0x7fffffffu];
    for (int q = b + 1; q < e; ++q) t = add_rn(t, w[idx[q] & 0x7fffffffu]);
    if (e - b <= 8) {
      // load every member's p and c before the first store of w
      unsigned mm[8];
      T pv[8], cv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < e - b) {
          mm[q] = idx[b + q];
          pv[q] = p[mm[q] & 0x7fffffffu];
          cv[q] = c[mm[q] & 0x7fffffffu];
        }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < e - b) {
          T v = fma_rn(T(0.1), pv[q], t);
          if (mm[q] & 0x80000000u) v = T(0);
          w[mm[q] & 0x7fffffffu] = v;
          part = fma_rn(mul_rn(v, cv[q]), pv[q], part);
        }
    } else {
      for (int q = b; q < e; ++q) {
        const unsigned m = idx[q];
        const unsigned id = m & 0x7fffffffu;
        const T pv = p[id];
        T v = fma_rn(T(0.1), pv, t);
        if (m & 0x80000000u) v = T(0);
        w[id] = v;
        part = fma_rn(mul_rn(v, c[id]), pv, part);
      }
    }
  }
  const double s = block_sum<T>(part, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block(counter, gridDim.x)) {
    const double s1 = block_sum_array(ax_partial, n_ax_partial, red);
    __syncthreads();
    const double s2 = block_sum_array(partial, gridDim.x, red);
    if (threadIdx.x == 0) {
      const double pap = s1 + s2;
      sc->pap = pap;
      sc->alpha = sc->rtz1 / pap;
    }
  }
}

// ------------------------------------------------- defect boundary pass --
// Boundary half of MODE 2: t = jl-order group sum of w_L; A x = t + 0.1 x
// (0 when masked); r = f - A x; r'Cr reduced with the interior partials into
// sc->rtr and sc->rnorm.
template <typename T>
__global__ void __launch_bounds__(256)
    k_gs_res(const T *__restrict__ w, const T *__restrict__ x,
             const T *__restrict__ f, T *__restrict__ r, const T *__restrict__ c,
             const int *__restrict__ off, const unsigned *__restrict__ idx, int ng,
             double *__restrict__ partial, const double *__restrict__ ax_partial,
             int n_ax_partial, unsigned *counter, CgScalars *sc) {
  __shared__ double red[32];
  T part = T(0);
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng;
       g += gridDim.x * blockDim.x) {
    const int b = off[g], e = off[g + 1];
    T t = w[idx[b] & 0x7fffffffu];
    for (int q = b + 1; q < e; ++q) t = add_rn(t, w[idx[q] & 0x7fffffffu]);
    if (e - b <= 8) {
      unsigned mm[8];
      T xv[8], fv[8], cv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < e - b) {
          mm[q] = idx[b + q];
          const unsigned id = mm[q] & 0x7fffffffu;
          xv[q] = x[id];
          fv[q] = f[id];
          cv[q] = c[id];
        }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < e - b) {
          T ax = fma_rn(T(0.1), xv[q], t);
          if (mm[q] & 0x80000000u) ax = T(0);
          const T rv = fv[q] - ax;
          r[mm[q] & 0x7fffffffu] = rv;
          part = fma_rn(mul_rn(rv, cv[q]), rv, part);
        }
    } else {
      for (int q = b; q < e; ++q) {
        const unsigned m = idx[q];
        const unsigned id = m & 0x7fffffffu;
        T ax = fma_rn(T(0.1), x[id], t);
        if (m & 0x80000000u) ax = T(0);
        const T rv = f[id] - ax;
        r[id] = rv;
        part = fma_rn(mul_rn(rv, c[id]), rv, part);
      }
    }
  }
  const double s = block_sum<T>(part, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block(counter, gridDim.x)) {
    const double s1 = block_sum_array(ax_partial, n_ax_partial, red);
    __syncthreads();
    const double s2 = block_sum_array(partial, gridDim.x, red);
    if (threadIdx.x == 0) {
      sc->rtr = s1 + s2;
      sc->rnorm = sqrt(s1 + s2);
    }
  }
}

// ------------------------------------------------------------ CG update --
// x += alpha p; r -= alpha w (add2s2, cg.f:63-64); rtr = glsc3(r,c,r) (cg.f:66).
// The last block forms rnorm and, for the identity preconditioner (z = r),
// the next rtz1 = rtr and beta = rtz1/rtz2 (cg.f:52-55).
// DEFER pairs the x updates of two iterations whose directions sit in two
// buffers: 1 leaves x alone and keeps alpha in sc->alpha_prev; 2 then makes
// x += alpha_prev pprev, x += alpha p, the two fused multiply-adds of the
// unpaired form in the same order (bitwise the same x), reading and writing
// x once for the two iterations.
// CF (FP32, even lx <= 16): c is the verified closed-form multiplicity
// (c_closed_form), 2^-m with m the number of the point's extreme local
// indices whose face has a neighbour (cface[e]: bit 0/1 the faces i = 0 /
// lx-1, 2/3 for j, 4/5 for k); the 16-byte path forms it instead of
// reading c (the same values, so the same rtr).
template <typename T, int DEFER = 0, bool CF = false>
__global__ void __launch_bounds__(256)
    k_cg_update(T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
                const T *__restrict__ w, const T *__restrict__ c, long n,
                double *__restrict__ partial, unsigned *counter, CgScalars *sc,
                double *hist, int iter, int identity_precond,
                float *__restrict__ r32 = nullptr, const T *__restrict__ pprev = nullptr,
                const unsigned char *__restrict__ cface = nullptr, int lx = 0) {
  __shared__ double red[32];
  // CF: the extreme-index bits of the four points of each 16-byte group
  // of an element, one byte a point
  __shared__ unsigned ext4[CF ? 1024 : 1];
  const T alpha = T(sc->alpha);
  const T alphm = -alpha;
  const T alpha0 = DEFER == 2 ? T(sc->alpha_prev) : T(0);
  if (DEFER == 1 && blockIdx.x == 0 && threadIdx.x == 0) sc->alpha_prev = sc->alpha;
  T part = T(0);
  // 16-byte loads and stores (two doubles or four floats a thread) when
  // every vector allows them
  constexpr int VEC = 16 / int(sizeof(T));
  typedef typename std::conditional<sizeof(T) == 8, double2, float4>::type V;
  const uintptr_t al = reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(r) |
                       reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(w) |
                       reinterpret_cast<uintptr_t>(c) |
                       (DEFER == 2 ? reinterpret_cast<uintptr_t>(pprev) : uintptr_t(0));
  const bool vec = (al & 15u) == 0 && n % VEC == 0 &&
                   (!r32 || (reinterpret_cast<uintptr_t>(r32) & uintptr_t(4 * VEC - 1)) == 0);
  // CF: element e and group l4 of v, advanced by the stride's quotient and
  // remainder
  long e = 0, se = 0;
  int l4 = 0, sl = 0;
  const int Q = CF ? lx * lx * lx / 4 : 1;
  if constexpr (CF) {
    const long v0 = long(blockIdx.x) * blockDim.x + threadIdx.x;
    const long vs = long(gridDim.x) * blockDim.x;
    static_assert(VEC == 4, "closed-form multiplicity: FP32 only");
    const int L2 = lx * lx;
    for (int t = threadIdx.x; t < Q; t += blockDim.x) {
      unsigned b4 = 0;
      for (int d = 0; d < 4; ++d) {
        const int l = 4 * t + d, i = l % lx, j = (l / lx) % lx, k = l / L2;
        const unsigned b = (i == 0 ? 1u : 0u) | (i == lx - 1 ? 2u : 0u) |
                           (j == 0 ? 4u : 0u) | (j == lx - 1 ? 8u : 0u) |
                           (k == 0 ? 16u : 0u) | (k == lx - 1 ? 32u : 0u);
        b4 |= b << (8 * d);
      }
      ext4[t] = b4;
    }
    __syncthreads();
    e = v0 / Q;
    l4 = int(v0 - e * Q);
    se = vs / Q;
    sl = int(vs - se * Q);
  }
  if (vec) {
    for (long v = long(blockIdx.x) * blockDim.x + threadIdx.x; v < n / VEC;
         v += long(gridDim.x) * blockDim.x) {
      alignas(16) T xa[VEC], ra[VEC], pa[VEC], wa[VEC], ca[VEC], qa[VEC];
      if (DEFER != 1) {
        *reinterpret_cast<V *>(xa) = reinterpret_cast<const V *>(x)[v];
        *reinterpret_cast<V *>(pa) = reinterpret_cast<const V *>(p)[v];
      }
      if (DEFER == 2) *reinterpret_cast<V *>(qa) = reinterpret_cast<const V *>(pprev)[v];
      *reinterpret_cast<V *>(ra) = reinterpret_cast<const V *>(r)[v];
      *reinterpret_cast<V *>(wa) = reinterpret_cast<const V *>(w)[v];
      if constexpr (CF) {
        const unsigned fb = __ldg(cface + e), b4 = ext4[l4];
#pragma unroll
        for (int q = 0; q < VEC; ++q)
          ca[q] = T(__int_as_float((127 - __popc((b4 >> (8 * q)) & fb)) << 23));
        l4 += sl;
        e += se;
        if (l4 >= Q) {
          l4 -= Q;
          ++e;
        }
      } else {
        *reinterpret_cast<V *>(ca) = reinterpret_cast<const V *>(c)[v];
      }
      alignas(16) float r3[VEC];
#pragma unroll
      for (int q = 0; q < VEC; ++q) {
        if (DEFER == 2) xa[q] = fma_rn(alpha0, qa[q], xa[q]);
        if (DEFER != 1) xa[q] = fma_rn(alpha, pa[q], xa[q]);
        ra[q] = fma_rn(alphm, wa[q], ra[q]);
        r3[q] = float(ra[q]);
        part = fma_rn(mul_rn(ra[q], ca[q]), ra[q], part);
      }
      if (DEFER != 1) reinterpret_cast<V *>(x)[v] = *reinterpret_cast<const V *>(xa);
      reinterpret_cast<V *>(r)[v] = *reinterpret_cast<const V *>(ra);
      if (r32) {
        if constexpr (VEC == 2)
          reinterpret_cast<float2 *>(r32)[v] = *reinterpret_cast<const float2 *>(r3);
        else
          reinterpret_cast<float4 *>(r32)[v] = *reinterpret_cast<const float4 *>(r3);
      }
    }
  } else {
    for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
         q += long(gridDim.x) * blockDim.x) {
      if (DEFER == 2) x[q] = fma_rn(alpha, p[q], fma_rn(alpha0, pprev[q], x[q]));
      else if (DEFER == 0) x[q] = fma_rn(alpha, p[q], x[q]);
      const T rv = fma_rn(alphm, w[q], r[q]);
      r[q] = rv;
      if (r32) r32[q] = float(rv);  // the FP32 V-cycle's input, as k_to_f32 makes it
      part = fma_rn(mul_rn(rv, c[q]), rv, part);
    }
  }
  const double s = block_sum<T>(part, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block(counter, gridDim.x)) {
    const double rtr = block_sum_array(partial, gridDim.x, red);
    if (threadIdx.x == 0) {
      sc->rtr = rtr;
      if (iter == 1) sc->rtr_first = rtr;
      sc->rnorm = sqrt(rtr);
      sc->iter = iter;
      if (hist) {
        double *h = hist + 5 * iter;
        h[0] = sc->rnorm;
        h[1] = sc->alpha;
        h[2] = sc->beta;
        h[3] = sc->pap;
        h[4] = sc->rtz1;
      }
      if (identity_precond) {
        sc->rtz2 = sc->rtz1;
        sc->rtz1 = rtr;
        sc->beta = sc->rtz1 / sc->rtz2;
      }
    }
  }
}

// ------------------------------------------------------------ reductions --
// s = glsc3(a,b,mult) (math.f:603-617) into *out via partials; optional
// CG bookkeeping: mode 1 = initial rnorm (cg.f:42), mode 2 = rtz1 and beta of
// a preconditioned iteration (cg.f:51-55).  With mf, the third vector is
// formed here from the FP32 vector mf (T(mf[q]), as k_to_f64 makes it) and
// stored to mout (m itself is not read).
template <typename T>
__global__ void __launch_bounds__(256)
    k_glsc3(const T *__restrict__ a, const T *__restrict__ b,
            const T *m, long n, double *__restrict__ partial,
            unsigned *counter, double *out, CgScalars *sc, int mode,
            double *hist, int iter, const float *__restrict__ mf = nullptr,
            T *mout = nullptr) {
  __shared__ double red[32];
  T part = T(0);
  // 16-byte accesses (two doubles or four floats a thread) when every vector
  // allows them
  constexpr int VEC = 16 / int(sizeof(T));
  typedef typename std::conditional<sizeof(T) == 8, double2, float4>::type V;
  typedef typename std::conditional<sizeof(T) == 8, float2, float4>::type VF;
  const uintptr_t al = reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                       reinterpret_cast<uintptr_t>(mf ? mout : m);
  const bool vec = (al & 15u) == 0 && n % VEC == 0 &&
                   (!mf || (reinterpret_cast<uintptr_t>(mf) & uintptr_t(4 * VEC - 1)) == 0);
  if (vec) {
    for (long v = long(blockIdx.x) * blockDim.x + threadIdx.x; v < n / VEC;
         v += long(gridDim.x) * blockDim.x) {
      alignas(16) T aa[VEC], ba[VEC], ma[VEC];
      *reinterpret_cast<V *>(aa) = reinterpret_cast<const V *>(a)[v];
      *reinterpret_cast<V *>(ba) = reinterpret_cast<const V *>(b)[v];
      if (mf) {
        alignas(16) float fa[VEC];
        *reinterpret_cast<VF *>(fa) = reinterpret_cast<const VF *>(mf)[v];
#pragma unroll
        for (int q = 0; q < VEC; ++q) ma[q] = T(fa[q]);
        reinterpret_cast<V *>(mout)[v] = *reinterpret_cast<const V *>(ma);
      } else {
        *reinterpret_cast<V *>(ma) = reinterpret_cast<const V *>(m)[v];
      }
#pragma unroll
      for (int q = 0; q < VEC; ++q) part = fma_rn(mul_rn(aa[q], ba[q]), ma[q], part);
    }
  } else {
    for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
         q += long(gridDim.x) * blockDim.x) {
      T mv;
      if (mf) {
        mv = T(mf[q]);
        mout[q] = mv;
      } else {
        mv = m[q];
      }
      part = fma_rn(mul_rn(a[q], b[q]), mv, part);
    }
  }
  const double s = block_sum<T>(part, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block(counter, gridDim.x)) {
    const double v = block_sum_array(partial, gridDim.x, red);
    if (threadIdx.x == 0) {
      if (out) *out = v;
      if (sc && mode == 1) {
        sc->rnorm = sqrt(v);
        sc->rtz1 = v;   // with z = r the first rtz1 equals this value
        sc->rtz2 = 1.0;
        sc->beta = 0.0;
        if (hist) {
          hist[0] = sc->rnorm;
          hist[1] = hist[2] = hist[3] = hist[4] = 0.0;
        }
      }
      if (sc && mode == 2) {
        sc->rtz2 = sc->rtz1;
        sc->rtz1 = v;
        sc->beta = (iter == 1) ? 0.0 : v / sc->rtz2;
      }
    }
  }
}

}  // namespace nb

#include "nb_tma.cuh"

namespace nb {

// ------------------------------------------- FP32 operator, TMA metric --
// The FP32 element operator with the element's whole metric block
// (24*lx1^3 bytes, contiguous in gxyz(6,nxyz,nelt)) brought into shared
// memory by one bulk copy issued when the CTA starts.  The copy overlaps the
// loads of z and the old p; the arithmetic is that of k_ax_impl<float,..,RD>
// (same order, same results).  Even lx1 only (the copy size must be a
// multiple of 16 bytes).
template <int LX>
struct AxTmaShared {
  alignas(128) float g[6 * LX * LX * LX];
  alignas(16) float u[LX * LX * LX];
  alignas(16) float wr[LX * LX * LX];
  alignas(16) float ws[LX * LX * LX];
  alignas(16) float Dr[LX * LX];
  alignas(16) float Dc[LX * LX];
  alignas(8) uint64_t bar;
  alignas(16) double red[32];
};

template <int LX, int MODE>
__global__ void __launch_bounds__(LX * LX)
    k_ax_f32_tma(AxArgs<float> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AxTmaShared<LX> &sm = *reinterpret_cast<AxTmaShared<LX> *>(smem_raw);
  constexpr int L2 = LX * LX, L3 = LX * LX * LX;
  constexpr unsigned GBYTES = 24u * L3;
  const int i = threadIdx.x, j = threadIdx.y;
  const int tid = i + LX * j;
  const int e = blockIdx.x;
  const size_t base = size_t(e) * L3;

  if (tid == 0) block_copy_begin(&sm.bar, sm.g, a.g + 6 * base, GBYTES, a.wait_test);
  {
    const int r = tid % LX, m = tid / LX;
    const float d = a.D[r + m * LX];
    sm.Dr[r * LX + m] = d;
    sm.Dc[m * LX + r] = d;
  }
  float ureg[LX];
  const bool col_interior = (i > 0) && (i < LX - 1) && (j > 0) && (j < LX - 1);
  float creg[LX];
  if (MODE == 1 && col_interior) {
#pragma unroll
    for (int k = 1; k < LX - 1; ++k)
      creg[k] = a.c_unit_interior ? 1.f : a.c[base + size_t(k) * L2 + tid];
  }
  float beta = 0.f;
  if (MODE == 1 && !a.first) beta = float(a.sc->beta);
  float pold[LX];
#pragma unroll
  for (int k = 0; k < LX; ++k) {  // all loads before the first store
    const size_t id = base + size_t(k) * L2 + tid;
    ureg[k] = a.u[id];
    pold[k] = (MODE == 1 && !a.first) ? a.pold[id] : 0.f;
  }
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + tid;
    if (MODE == 1) {
      if (!a.first) ureg[k] = fma_rn(beta, pold[k], ureg[k]);
      a.p[id] = ureg[k];
    }
    sm.u[k * L2 + tid] = ureg[k];
  }
  __syncthreads();
  float Di[LX], Dj[LX];
#pragma unroll
  for (int m = 0; m < LX; ++m) {
    Di[m] = sm.Dr[i * LX + m];
    Dj[m] = sm.Dr[j * LX + m];
  }
  if (!block_copy_wait(&sm.bar, a.err, a.wait_test, sm.red, a.g)) return;

  float wtreg[LX];
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const float *urow = &sm.u[k * L2 + j * LX];
    const float *ucol = &sm.u[k * L2 + i];
    const float ur = dot_contig<float, LX>(Di, urow);
    float us = mul_rn(ucol[0], Dj[0]);
#pragma unroll
    for (int m = 1; m < LX; ++m) us = fma_rn(ucol[m * LX], Dj[m], us);
    const float ut = dot_contig<float, LX>(ureg, &sm.Dr[k * LX]);
    const float2 *gp = reinterpret_cast<const float2 *>(&sm.g[6 * (k * L2 + tid)]);
    const float2 g01 = gp[0], g23 = gp[1], g45 = gp[2];
    float wr = mul_rn(g01.x, ur);
    wr = fma_rn(g01.y, us, wr);
    wr = fma_rn(g23.x, ut, wr);
    float ws = mul_rn(g01.y, ur);
    ws = fma_rn(g23.y, us, ws);
    ws = fma_rn(g45.x, ut, ws);
    float wt = mul_rn(g23.x, ur);
    wt = fma_rn(g45.x, us, wt);
    wt = fma_rn(g45.y, ut, wt);
    sm.wr[k * L2 + tid] = wr;
    sm.ws[k * L2 + tid] = ws;
    wtreg[k] = wt;
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < LX; ++m) {
    Di[m] = sm.Dc[i * LX + m];
    Dj[m] = sm.Dc[j * LX + m];
  }
  float part = 0.f;
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const float *rrow = &sm.wr[k * L2 + j * LX];
    const float *scol = &sm.ws[k * L2 + i];
    const float tr = dot_contig<float, LX>(Di, rrow);
    float ts = mul_rn(scol[0], Dj[0]);
#pragma unroll
    for (int m = 1; m < LX; ++m) ts = fma_rn(scol[m * LX], Dj[m], ts);
    const float tt = dot_contig<float, LX>(wtreg, &sm.Dc[k * LX]);
    float wl = add_rn(add_rn(tr, ts), tt);
    const size_t id = base + size_t(k) * L2 + tid;
    if (MODE == 1) {
      if (col_interior && k > 0 && k < LX - 1) {
        wl = fma_rn(0.1f, ureg[k], wl);
        part = fma_rn(mul_rn(wl, creg[k]), ureg[k], part);
      }
    }
    a.w[id] = wl;
  }
  if (MODE == 1) {
    const double s = block_sum<float>(part, sm.red);
    if (i == 0 && j == 0) a.partial[e] = s;
  }
}

template <int LX>
constexpr size_t ax_tma_smem_bytes() {
  return sizeof(AxTmaShared<LX>);
}

}  // namespace nb

namespace nb {

// ------------------------------------------ FP64 operator, even-odd split --
// The GLL derivative matrix is anti-centrosymmetric, D(n-1-i,n-1-m) =
// -D(i,m) (n = lx1, even here), so each 1-D contraction y = D v splits into
// an even and an odd half (Solomonoff's even-odd decomposition):
//   ve(m) = v(m) + v(n-1-m),  vo(m) = v(m) - v(n-1-m),          m < n/2
//   ye(a) = sum_m E(a,m) ve(m), yo(a) = sum_m O(a,m) vo(m),      a < n/2
//   y(a) = ye(a) + yo(a),   y(n-1-a) = yo(a) - ye(a)
// with E(a,m) = (D(a,m) + D(a,n-1-m))/2, O(a,m) = (D(a,m) - D(a,n-1-m))/2.
// Per output that is n/2 fused multiply-adds plus two additions instead of n
// multiply-adds: the FP64 pipe, which bounds this kernel on GB300, does ~27%
// less work per point.  Sums are taken in a different order from the
// reference's left-to-right mxm, so results agree with it to rounding, not
// bit for bit (the reference-order kernel stays available).
//
// One CTA per element, lx1*lx1 threads.  Thread t owns, in turn, the line
// (j,k)=(t%n,t/n) of the r contraction, the line (i,k) of the s contraction
// and its own column (i,j) of the t contraction (kept in registers).
// Shared arrays use a row pitch of n+1 doubles (bank-conflict free lines).
// TMAG: the element's metric block (6*lx1^3 values, contiguous in
// gxyz(6,nxyz,nelt)) arrives in shared memory by one bulk copy issued when
// the CTA starts, instead of per-point loads in the metric step -- the FP32
// form, where those loads would otherwise wait on DRAM latency one plane at
// a time.
// Shared-memory layout of the even-odd kernels.  The FP32 forms up to
// lx1 = 12 keep rows unpadded, so a warp's column accesses (7 per point)
// touch 32 consecutive words, and space the planes eo_plane words apart;
// their r- and s-line phases take the lines in the order of EoCoef's maps,
// which deal each warp lines that start in distinct banks.  The other forms
// pad rows to lx1 + 1 and take lines in natural order.
template <typename T, int LX>
constexpr bool eo_dealt() { return sizeof(T) == 4 && LX <= 12; }

template <typename T, int LX>
constexpr int eo_plane() {
  if constexpr (eo_dealt<T, LX>()) {
    // plane strides with the fewest conflicts of the dealt lines
    return LX == 12 ? 145 : LX == 10 ? 103 : LX == 8 ? 71 : LX == 6 ? 47 : LX == 4 ? 19 : LX * LX;
  } else {
    return (LX + 1) * LX;
  }
}

template <typename T, int LX>
__device__ __forceinline__ int eo_at(int i, int j, int k) {
  return i + (eo_dealt<T, LX>() ? LX : LX + 1) * j + eo_plane<T, LX>() * k;
}

template <typename T, int LX, bool TMAG>
struct AxEoShared {
  static constexpr int N = eo_plane<T, LX>() * LX;
  alignas(128) T g[TMAG ? 6 * LX * LX * LX : 2];
  T A[N];
  T B[N];
  T C[N];
  T E4[4 * (LX / 2) * (LX / 2)];  // E, O of D, then E, O of D^T
  alignas(8) uint64_t bar;
  alignas(16) double red[32];
};


// y(0..n-1) of a folded line v (length n), coefficients Ec/Oc (h x h, row a)
template <typename T, int LX>
__device__ __forceinline__ void eo_line(const T *v, const T *Ec, const T *Oc, T *y) {
  constexpr int H = LX / 2;
  T ve[H], vo[H];
#pragma unroll
  for (int m = 0; m < H; ++m) {
    ve[m] = add_rn(v[m], v[LX - 1 - m]);
    vo[m] = v[m] - v[LX - 1 - m];
  }
#pragma unroll
  for (int a = 0; a < H; ++a) {
    T ye = mul_rn(Ec[a * H], ve[0]);
    T yo = mul_rn(Oc[a * H], vo[0]);
#pragma unroll
    for (int m = 1; m < H; ++m) {
      ye = fma_rn(Ec[a * H + m], ve[m], ye);
      yo = fma_rn(Oc[a * H + m], vo[m], yo);
    }
    y[a] = add_rn(ye, yo);
    y[LX - 1 - a] = yo - ye;
  }
}

// The even-odd tables (E, O of D, then E, O of D^T; 4*(lx1/2)^2 values) as
// a kernel parameter.  Every lane reads the same coefficient at the same
// time, so from the parameter bank they are operands of the FMAs
// themselves; from shared memory each one was a broadcast load.
// rmap / smap (FP32 forms up to lx1 = 12): the r-line (j, k) and s-line
// (i, k) that thread t takes, as j + lx1 k and i + lx1 k (eo_line_maps).
template <typename T, int LX>
struct EoCoef {
  T c[4 * (LX / 2) * (LX / 2)];
  unsigned char rmap[LX * LX], smap[LX * LX];
};

// The line maps of an lx1^2-thread CTA whose planes are pl words apart
// (nb_solver.cu).
void eo_line_maps(int lx, int pl, unsigned char *rmap, unsigned char *smap);

// A launch's EoCoef: the tables eo (FP64, host) rounded to T, and the line
// maps of the form's layout (identity for the forms that do not deal lines).
template <typename T, int LX>
void eo_fill(EoCoef<T, LX> &cf, const double *eo) {
  struct Maps {
    unsigned char r[LX * LX], s[LX * LX];
    Maps() {
      if (eo_dealt<T, LX>()) {
        eo_line_maps(LX, eo_plane<T, LX>(), r, s);
      } else {
        for (int t = 0; t < LX * LX; ++t) r[t] = s[t] = (unsigned char)t;
      }
    }
  };
  static const Maps maps;
  for (int q = 0; q < 4 * (LX / 2) * (LX / 2); ++q) cf.c[q] = T(eo[q]);
  for (int t = 0; t < LX * LX; ++t) {
    cf.rmap[t] = maps.r[t];
    cf.smap[t] = maps.s[t];
  }
}

template <typename T, int LX, int MODE, bool TMAG>
__device__ __forceinline__ void ax_eo_body(const AxArgs<T> &a, const EoCoef<T, LX> &cf);

template <typename T, int LX, int MODE, bool TMAG>
__global__ void __launch_bounds__(LX * LX)
    k_ax_eo(AxArgs<T> a, const __grid_constant__ EoCoef<T, LX> cf) {
  ax_eo_body<T, LX, MODE, TMAG>(a, cf);
}
// The same with four CTAs per SM asked for (the FP64 lx1 = 12 operator):
// the FP64 pipe is its bound, and a fourth CTA's warps cover the barrier
// and shared-memory waits
template <typename T, int LX, int MODE, bool TMAG>
__global__ void __launch_bounds__(LX * LX, 4)
    k_ax_eo4(AxArgs<T> a, const __grid_constant__ EoCoef<T, LX> cf) {
  ax_eo_body<T, LX, MODE, TMAG>(a, cf);
}

template <typename T, int LX, int MODE, bool TMAG>
__device__ __forceinline__ void ax_eo_body(const AxArgs<T> &a, const EoCoef<T, LX> &cf) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AxEoShared<T, LX, TMAG> &sm = *reinterpret_cast<AxEoShared<T, LX, TMAG> *>(smem_raw);
  constexpr int L2 = LX * LX, L3 = LX * LX * LX, H = LX / 2;
  const int t = threadIdx.x + LX * threadIdx.y;
  const int i = threadIdx.x, j = threadIdx.y;  // own column (i,j)
  const int e = blockIdx.x;
  const size_t base = size_t(e) * L3;
  // the element's metric block (the shared one when all blocks are equal)
  const T *gblk = a.g + (a.g_uniform ? size_t(0) : 6 * base);
  if (TMAG && t == 0)
    block_copy_begin(&sm.bar, sm.g, gblk, unsigned(6 * L3 * sizeof(T)), a.wait_test);
  // FP32 up to lx1 = 12 reads the coefficients from the parameter bank.
  // FP64 and the larger FP32 shapes copy them to shared memory: from the
  // parameter bank the compiler keeps many of them in registers, and those
  // forms spill (FP64) or double their registers (FP32, lx1 = 16).
  constexpr bool CPAR = sizeof(T) == 4 && LX <= 12;
  if constexpr (!CPAR)
    for (int q = t; q < 4 * H * H; q += L2) sm.E4[q] = cf.c[q];
  const T *E4 = CPAR ? cf.c : sm.E4;
  const T *Ed = E4, *Od = E4 + H * H;                // of D
  const T *Et = E4 + 2 * H * H, *Ot = E4 + 3 * H * H;  // of D^T

  // the r-line (r0 = j, r1 = k) and s-line (s0 = i, s1 = k) of this thread
  constexpr bool DEALT = eo_dealt<T, LX>();
  const int lr = DEALT ? int(cf.rmap[t]) : t, ls = DEALT ? int(cf.smap[t]) : t;
  const int r0 = lr % LX, r1 = lr / LX, s0 = ls % LX, s1 = ls / LX;

  const bool col_interior = (i > 0) && (i < LX - 1) && (j > 0) && (j < LX - 1);
  T creg[LX], freg[LX];
  if (MODE != 0 && col_interior) {
#pragma unroll
    for (int k = 1; k < LX - 1; ++k) {
      const size_t id = base + size_t(k) * L2 + t;
      creg[k] = (MODE == 1 && a.c_unit_interior) ? T(1) : a.c[id];
      if (MODE == 2) freg[k] = a.f[id];
    }
  }
  T ureg[LX], pold[LX];
  const T beta = (MODE == 1 && !a.first) ? T(a.sc->beta) : T(0);
#pragma unroll
  for (int k = 0; k < LX; ++k) {  // all loads before the first store
    const size_t id = base + size_t(k) * L2 + t;
    if (MODE == 1) {
      ureg[k] = a.u[id];
      pold[k] = a.first ? T(0) : a.pold[id];
    } else if (MODE == 2) {
      ureg[k] = a.p[id];
      pold[k] = a.e ? T(a.e[id]) : T(0);
    } else {
      ureg[k] = a.u[id];
    }
  }
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const size_t id = base + size_t(k) * L2 + t;
    if (MODE == 1) {
      if (!a.first) ureg[k] = fma_rn(beta, pold[k], ureg[k]);  // add2s1, math.f:534
      a.p[id] = ureg[k];
    } else if (MODE == 2 && a.e) {
      ureg[k] = fma_rn(T(a.scale), pold[k], ureg[k]);
      a.p[id] = ureg[k];
    }
    sm.A[eo_at<T, LX>(i, j, k)] = ureg[k];
  }
  __syncthreads();

  // gradient (local_grad3, cg.f:170-187) as three folded contractions
  {
    T v[LX], y[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.A[eo_at<T, LX>(m, r0, r1)];  // line (j,k)
    eo_line<T, LX>(v, Ed, Od, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.B[eo_at<T, LX>(m, r0, r1)] = y[m];  // ur
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.A[eo_at<T, LX>(s0, m, s1)];  // line (i,k)
    eo_line<T, LX>(v, Ed, Od, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.C[eo_at<T, LX>(s0, m, s1)] = y[m];  // us
  }
  T wtreg[LX];
  eo_line<T, LX>(ureg, Ed, Od, wtreg);  // ut of the own column
  __syncthreads();

  // metric, cg.f:156-163 (wr, ws back into B, C; wt in registers)
  if (TMAG && !block_copy_wait(&sm.bar, a.err, a.wait_test, sm.red, gblk)) return;
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const int q = eo_at<T, LX>(i, j, k);
    const T ur = sm.B[q], us = sm.C[q], ut = wtreg[k];
    typedef typename Vec2<T>::type V2;
    const V2 *gp = TMAG ? reinterpret_cast<const V2 *>(&sm.g[6 * (k * L2 + t)])
                        : reinterpret_cast<const V2 *>(gblk + 6 * (k * L2 + t));
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

  // transposed gradient (local_grad3_t, cg.f:189-212) with D^T
  {
    T v[LX], y[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.B[eo_at<T, LX>(m, r0, r1)];  // wr line (j,k)
    eo_line<T, LX>(v, Et, Ot, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.A[eo_at<T, LX>(m, r0, r1)] = y[m];  // tr
  }
  __syncthreads();
  {
    T v[LX], y[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.C[eo_at<T, LX>(s0, m, s1)];  // ws line (i,k)
    eo_line<T, LX>(v, Et, Ot, y);
#pragma unroll
    for (int m = 0; m < LX; ++m) sm.B[eo_at<T, LX>(s0, m, s1)] = y[m];  // ts
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
    } else if (MODE == 2) {
      if (interior) {
        const T rv = freg[k] - fma_rn(T(0.1), ureg[k], wl);
        a.r[id] = rv;
        part = fma_rn(mul_rn(rv, creg[k]), rv, part);
      } else {
        a.w[id] = wl;
      }
    } else {
      a.w[id] = wl;
    }
  }
  if (MODE != 0) {
    const double s = block_sum<T>(part, sm.red);
    if (t == 0) a.partial[e] = s;
  }
}

template <typename T, int LX, bool TMAG>
constexpr size_t ax_eo_smem_bytes() {
  return sizeof(AxEoShared<T, LX, TMAG>);
}

}  // namespace nb

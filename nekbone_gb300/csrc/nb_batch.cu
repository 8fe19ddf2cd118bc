// nb_batch.cu -- many independent box-mesh Poisson problems solved together.
//
// Every problem is a brick of nelx*nely*nelz elements with its own lx1, the
// reference's numbering (set_vert_box, prox_dssum.f:42-73), the undeformed
// metric (setup_g, prox_setup.f:27-52), the full Dirichlet mask and a
// seeded uniform right-hand side.  The solver is the mixed one of a single
// mesh -- FP32 inner CG (cg.f:48-75 with z = r, fixed inner iterations)
// inside FP64 defect correction to |r|_C / |f|_C <= tol -- run for all
// problems at once:
//
//   * all problems' points, elements and element-boundary groups are
//     concatenated, problems ordered by lx1 so that each lx1 is one element
//     range (one launch of the batched element operator per lx1);
//   * the gather-scatter, vector and norm kernels work on chunks that never
//     straddle a problem; each chunk writes one partial, and the chunk that
//     arrives last for its problem (a per-problem counter) sums that
//     problem's partials in a fixed order, so every per-problem scalar is
//     deterministic;
//   * converged problems drop out (every kernel skips their chunks);
//   * the whole solve -- initial norms, then cycles of [scale, inner CG,
//     FP64 defect, convergence test] -- is one CUDA graph: the cycle is the
//     body of a conditional WHILE node whose condition a one-block kernel
//     sets from the problems' active flags (and a cycle bound), so a single
//     graph launch runs the solve to the end with no host round trip.
//
// The shape of the element operator per lx1 (elements per block and the D
// operand form) is chosen by nb_batch_tune, which times every instantiated
// shape on the batch's own elements.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/nekbone_gb300.h"
#include "nb_batch.h"
#include "nb_solver.h"

namespace nb {

cudaStream_t lib_stream();

namespace {

// Boundary groups per chunk (one CTA; a chunk never straddles a problem):
// eight per thread.  With one group per thread the per-CTA reductions and
// counters dominated: the inner boundary phase of the 256-problem workload
// took 126 ms (166 ms as a loop), 94-96 ms with 2048-8192 per chunk.
#ifndef NB_BATCH_GROUP_CHUNK
#define NB_BATCH_GROUP_CHUNK 2048
#endif
constexpr int kGroupChunk = NB_BATCH_GROUP_CHUNK;
constexpr int kPointChunk = 2048;  // points per chunk, eight per thread
constexpr int kThreads = 256;

// ------------------------------------------------------------- kernels --
// Boundary groups of the inner FP32 iteration (k_gs_fin per problem): w =
// jl-order group sum of w_L + 0.1 p (0 when masked), the boundary part of
// pap; the problem's last chunk forms pap and alpha = rtz1 / pap.
__global__ void __launch_bounds__(kThreads)
    k_bgs_fin(float *__restrict__ w, const float *__restrict__ p, const float *__restrict__ c,
              const int *__restrict__ off, const unsigned *__restrict__ idx,
              const int *__restrict__ gch_g0, const int *__restrict__ gch_prob,
              const BatchProb *__restrict__ pb, BatchScalars *sc, double *__restrict__ part_gs,
              const double *__restrict__ part_ax, unsigned *cnt) {
  __shared__ double red[32];
  const int ch = blockIdx.x;
  const int prob = gch_prob[ch];
  if (!sc[prob].active || !sc[prob].iactive) return;
  float part = 0.f;
  const int gend = gch_g0[ch + 1];
  for (int g = gch_g0[ch] + threadIdx.x; g < gend; g += kThreads) {
    const int b = off[g], e = off[g + 1];
    float t = w[idx[b] & 0x7fffffffu];
    for (int q = b + 1; q < e; ++q) t = add_rn(t, w[idx[q] & 0x7fffffffu]);
    unsigned mm[8];
    float pv[8], cv[8];
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
        float v = fma_rn(0.1f, pv[q], t);
        if (mm[q] & 0x80000000u) v = 0.f;
        w[mm[q] & 0x7fffffffu] = v;
        part = fma_rn(mul_rn(v, cv[q]), pv[q], part);
      }
  }
  const double s = block_sum<float>(part, red);
  if (threadIdx.x == 0) part_gs[ch] = s;
  const BatchProb P = pb[prob];
  if (last_block(cnt + prob, P.ngc)) {
    const double s1 = block_sum_array(part_ax + P.el0, P.nelt, red);
    __syncthreads();
    const double s2 = block_sum_array(part_gs + P.gc0, P.ngc, red);
    if (threadIdx.x == 0) {
      const double pap = s1 + s2;
      sc[prob].pap = pap;
      sc[prob].alpha = pap != 0.0 ? sc[prob].rtz1 / pap : 0.0;
    }
  }
}

// Boundary groups of the FP64 defect: A x = group sum + 0.1 x (0 when
// masked), r = f - A x, boundary part of r'Cr; the problem's last chunk
// forms |r|_C, counts the cycle and decides whether the problem goes on.
__global__ void __launch_bounds__(kThreads)
    k_bgs_res(const double *__restrict__ w, const double *__restrict__ x,
              const double *__restrict__ f, double *__restrict__ r, const double *__restrict__ c,
              const int *__restrict__ off, const unsigned *__restrict__ idx,
              const int *__restrict__ gch_g0, const int *__restrict__ gch_prob,
              const BatchProb *__restrict__ pb, BatchScalars *sc, double *__restrict__ part_gs,
              const double *__restrict__ part_ax, unsigned *cnt, double tol, int max_outer) {
  __shared__ double red[32];
  const int ch = blockIdx.x;
  const int prob = gch_prob[ch];
  if (!sc[prob].active) return;
  double part = 0.0;
  const int gend = gch_g0[ch + 1];
  for (int g = gch_g0[ch] + threadIdx.x; g < gend; g += kThreads) {
    const int b = off[g], e = off[g + 1];
    double t = w[idx[b] & 0x7fffffffu];
    for (int q = b + 1; q < e; ++q) t = add_rn(t, w[idx[q] & 0x7fffffffu]);
    unsigned mm[8];
    double xv[8], fv[8], cv[8];
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
        double ax = fma_rn(0.1, xv[q], t);
        if (mm[q] & 0x80000000u) ax = 0.0;
        const double rv = fv[q] - ax;
        r[mm[q] & 0x7fffffffu] = rv;
        part = fma_rn(mul_rn(rv, cv[q]), rv, part);
      }
  }
  const double s = block_sum<double>(part, red);
  if (threadIdx.x == 0) part_gs[ch] = s;
  const BatchProb P = pb[prob];
  if (last_block(cnt + prob, P.ngc)) {
    const double s1 = block_sum_array(part_ax + P.el0, P.nelt, red);
    __syncthreads();
    const double s2 = block_sum_array(part_gs + P.gc0, P.ngc, red);
    if (threadIdx.x == 0) {
      BatchScalars &S = sc[prob];
      S.rtr = s1 + s2;
      S.rn = sqrt(s1 + s2);
      S.outer += 1;
      const bool converged = S.rn <= tol * S.rn0;
      S.active = (!converged && S.outer < max_outer) ? 1 : 0;
    }
  }
}

// Each element's face bits (cface: bit 0/1 the faces i = 0 / lx1-1 have a
// neighbour, 2/3 for j, 4/5 for k; read from c at the face points (1,1),
// 1/2 with a neighbour), and *ok cleared when any point's c differs bitwise
// from 2^-m, m the number of its extreme local indices on faces with a
// neighbour: the form k_bupd makes c in.  One block per element at a time.
__global__ void k_bc_closed_form(const float *__restrict__ c, const int *__restrict__ el_prob,
                                 const BatchProb *__restrict__ pb, int nelt,
                                 unsigned char *__restrict__ cface, int *ok) {
  __shared__ unsigned fb_s;
  for (int e = blockIdx.x; e < nelt; e += gridDim.x) {
    const BatchProb &P = pb[el_prob[e]];
    const int lx = P.lx, L2 = lx * lx, L3 = L2 * lx;
    const float *ce = c + P.pt0 + long(e - P.el0) * L3;
    if (threadIdx.x == 0) {
      const int m = 1, h = lx - 1;
      const int pt[6] = {0 + lx * m + L2 * m, h + lx * m + L2 * m, m + 0 + L2 * m,
                         m + lx * h + L2 * m, m + lx * m + 0,  m + lx * m + L2 * h};
      unsigned fb = 0;
      for (int f = 0; f < 6; ++f)
        if (ce[pt[f]] == 0.5f) fb |= 1u << f;
      fb_s = fb;
      cface[e] = (unsigned char)fb;
    }
    __syncthreads();
    const unsigned fb = fb_s;
    bool good = true;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
      const int i = l % lx, j = (l / lx) % lx, k = l / L2;
      const unsigned b = (i == 0 ? 1u : 0u) | (i == lx - 1 ? 2u : 0u) | (j == 0 ? 4u : 0u) |
                         (j == lx - 1 ? 8u : 0u) | (k == 0 ? 16u : 0u) |
                         (k == lx - 1 ? 32u : 0u);
      good &= __float_as_uint(ce[l]) == unsigned(127 - __popc(b & fb)) << 23;
    }
    // (also keeps the next element's fb_s write behind every read of this one)
    if (!__syncthreads_and(good) && threadIdx.x == 0) atomicExch(ok, 0);
  }
}

// The extreme-index bits of the points of one element of lx1 points a
// direction, four points (one byte each: bit 0/1 i = 0 / lx1-1, 2/3 for j,
// 4/5 for k) a word
std::vector<unsigned> ext_table(int lx) {
  const int L2 = lx * lx, Q4 = L2 * lx / 4;
  std::vector<unsigned> t(Q4, 0u);
  for (int q = 0; q < Q4; ++q)
    for (int d = 0; d < 4; ++d) {
      const int l = 4 * q + d, i = l % lx, j = (l / lx) % lx, k = l / L2;
      const unsigned b = (i == 0 ? 1u : 0u) | (i == lx - 1 ? 2u : 0u) | (j == 0 ? 4u : 0u) |
                         (j == lx - 1 ? 8u : 0u) | (k == 0 ? 16u : 0u) |
                         (k == lx - 1 ? 32u : 0u);
      t[q] |= b << (8 * d);
    }
  return t;
}

// Inner FP32 update (k_cg_update per problem): x += alpha p, r -= alpha w,
// r'Cr; the problem's last chunk forms rtz1 and beta (z = r), counts the
// iteration and, with itol > 0, ends the problem's inner CG of this cycle
// once r'Cr <= itol^2 of the cycle's first (it: the iteration within the
// cycle, at most max_inner).
// With cface (c verified as each problem's inverse multiplicity,
// k_bc_closed_form), the 16-byte paths form c = 2^-m from the element's
// face bits and the extreme-index bits of the point (ext4: four points a
// word, one table per lx1 at P.ext0) instead of reading it: the same values.
// DEFER pairs the x updates of two iterations whose directions sit in two
// buffers (as k_cg_update): 1 leaves x alone, keeps alpha in alpha_prev
// and marks the problem pending if its inner CG stops here (k_bflush then
// makes the update); 2 makes x += alpha_prev pprev, x += alpha p, the
// unpaired form's two fused multiply-adds in order.
template <int DEFER>
__global__ void __launch_bounds__(kThreads)
    k_bupd(float *__restrict__ x, float *__restrict__ r, const float *__restrict__ p,
           const float *__restrict__ w, const float *__restrict__ c,
           const long *__restrict__ pch_q0, const int *__restrict__ pch_prob,
           const BatchProb *__restrict__ pb, BatchScalars *sc, double *__restrict__ part_pt,
           unsigned *cnt, int it, int max_inner, double itol,
           const unsigned char *__restrict__ cface, const unsigned *__restrict__ ext4,
           const float *__restrict__ pprev) {
  __shared__ double red[32];
  const int ch = blockIdx.x;
  const int prob = pch_prob[ch];
  if (!sc[prob].active || !sc[prob].iactive) return;
  const float alpha = float(sc[prob].alpha);
  const float alphm = -alpha;
  const float alpha0 = DEFER == 2 ? float(sc[prob].alpha_prev) : 0.f;
  const long q0 = pch_q0[ch], q1 = pch_q0[ch + 1];
  float part = 0.f;
  const uintptr_t al = reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(r) |
                       reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(w) |
                       reinterpret_cast<uintptr_t>(c) |
                       (DEFER == 2 ? reinterpret_cast<uintptr_t>(pprev) : uintptr_t(0));
  if ((al & 15u) == 0 && ((q0 | q1) & 3) == 0) {
    // 16-byte accesses: chunk bounds are multiples of 4 (every lx1^3 of an
    // even lx1 is).  With cface: element le of the problem and group l4 of
    // v, advanced by the stride's quotient and remainder.
    const BatchProb P = pb[prob];
    const int Q4 = P.lx * P.lx * P.lx / 4;
    long le = 0;
    int l4 = 0, se = 0, sl = 0;
    if (cface) {
      const long vrel = (q0 - P.pt0) / 4 + threadIdx.x;
      le = vrel / Q4;
      l4 = int(vrel - le * Q4);
      se = kThreads / Q4;
      sl = kThreads - se * Q4;
    }
    for (long v = q0 / 4 + threadIdx.x; v < q1 / 4; v += kThreads) {
      float4 xv = make_float4(0.f, 0.f, 0.f, 0.f), pv = xv, qv = xv, cv = xv;
      if (DEFER != 1) {
        pv = reinterpret_cast<const float4 *>(p)[v];
        xv = reinterpret_cast<const float4 *>(x)[v];
      }
      if (DEFER == 2) qv = reinterpret_cast<const float4 *>(pprev)[v];
      const float4 wv = reinterpret_cast<const float4 *>(w)[v];
      float4 rv = reinterpret_cast<const float4 *>(r)[v];
      if (cface) {
        const unsigned fb = __ldg(cface + P.el0 + le), b4 = __ldg(ext4 + P.ext0 + l4);
        cv.x = __int_as_float((127 - __popc(b4 & fb)) << 23);
        cv.y = __int_as_float((127 - __popc((b4 >> 8) & fb)) << 23);
        cv.z = __int_as_float((127 - __popc((b4 >> 16) & fb)) << 23);
        cv.w = __int_as_float((127 - __popc((b4 >> 24) & fb)) << 23);
        l4 += sl;
        le += se;
        if (l4 >= Q4) {
          l4 -= Q4;
          ++le;
        }
      } else {
        cv = reinterpret_cast<const float4 *>(c)[v];
      }
      if (DEFER == 2) {
        xv.x = fma_rn(alpha0, qv.x, xv.x);
        xv.y = fma_rn(alpha0, qv.y, xv.y);
        xv.z = fma_rn(alpha0, qv.z, xv.z);
        xv.w = fma_rn(alpha0, qv.w, xv.w);
      }
      if (DEFER != 1) {
        xv.x = fma_rn(alpha, pv.x, xv.x);
        xv.y = fma_rn(alpha, pv.y, xv.y);
        xv.z = fma_rn(alpha, pv.z, xv.z);
        xv.w = fma_rn(alpha, pv.w, xv.w);
      }
      rv.x = fma_rn(alphm, wv.x, rv.x);
      rv.y = fma_rn(alphm, wv.y, rv.y);
      rv.z = fma_rn(alphm, wv.z, rv.z);
      rv.w = fma_rn(alphm, wv.w, rv.w);
      if (DEFER != 1) reinterpret_cast<float4 *>(x)[v] = xv;
      reinterpret_cast<float4 *>(r)[v] = rv;
      part = fma_rn(mul_rn(rv.x, cv.x), rv.x, part);
      part = fma_rn(mul_rn(rv.y, cv.y), rv.y, part);
      part = fma_rn(mul_rn(rv.z, cv.z), rv.z, part);
      part = fma_rn(mul_rn(rv.w, cv.w), rv.w, part);
    }
  } else {
#pragma unroll 4
    for (long q = q0 + threadIdx.x; q < q1; q += kThreads) {
      const float wv = w[q], rv0 = r[q], cv = c[q];
      if (DEFER == 2) x[q] = fma_rn(alpha, p[q], fma_rn(alpha0, pprev[q], x[q]));
      else if (DEFER == 0) x[q] = fma_rn(alpha, p[q], x[q]);
      const float rv = fma_rn(alphm, wv, rv0);
      r[q] = rv;
      part = fma_rn(mul_rn(rv, cv), rv, part);
    }
  }
  const double s = block_sum<float>(part, red);
  if (threadIdx.x == 0) part_pt[ch] = s;
  const BatchProb P = pb[prob];
  if (last_block(cnt + prob, P.npc)) {
    const double rtr = block_sum_array(part_pt + P.pc0, P.npc, red);
    if (threadIdx.x == 0) {
      BatchScalars &S = sc[prob];
      S.rtr = rtr;
      S.rtz2 = S.rtz1;
      S.rtz1 = rtr;
      S.beta = S.rtz2 != 0.0 ? S.rtz1 / S.rtz2 : 0.0;
      S.inner += 1;
      const bool stop = it >= max_inner || (itol > 0.0 && rtr <= itol * itol * S.irtr0);
      if (stop) S.iactive = 0;
      if (DEFER == 1) {
        S.alpha_prev = S.alpha;
        S.pend = stop ? 1 : 0;
      }
    }
  }
}

// The deferred x update of every problem whose inner CG stopped on the
// first iteration of a pair (pend): x += alpha_prev p, p the direction
// buffer of odd iterations.  Before the defect, which reads x.
__global__ void __launch_bounds__(kThreads)
    k_bflush(float *__restrict__ x, const float *__restrict__ p,
             const long *__restrict__ pch_q0, const int *__restrict__ pch_prob,
             const BatchScalars *__restrict__ sc) {
  const int ch = blockIdx.x;
  const int prob = pch_prob[ch];
  if (!sc[prob].active || !sc[prob].pend) return;
  const float alpha = float(sc[prob].alpha_prev);
  const long q0 = pch_q0[ch], q1 = pch_q0[ch + 1];
  for (long q = q0 + threadIdx.x; q < q1; q += kThreads) x[q] = fma_rn(alpha, p[q], x[q]);
}

// Start of a cycle: inner right-hand side r32 = r / |r|, inner x = 0, and
// the inner rtz1 = r32'C r32.
__global__ void __launch_bounds__(kThreads)
    k_bscale(float *__restrict__ r32, float *__restrict__ e32, const double *__restrict__ r,
             const float *__restrict__ c32, const long *__restrict__ pch_q0,
             const int *__restrict__ pch_prob, const BatchProb *__restrict__ pb,
             BatchScalars *sc, double *__restrict__ part_pt, unsigned *cnt) {
  __shared__ double red[32];
  const int ch = blockIdx.x;
  const int prob = pch_prob[ch];
  if (!sc[prob].active) return;
  const double inv = 1.0 / sc[prob].rn;
  const long q0 = pch_q0[ch], q1 = pch_q0[ch + 1];
  float part = 0.f;
#pragma unroll 4
  for (long q = q0 + threadIdx.x; q < q1; q += kThreads) {
    const float v = float(r[q] * inv);
    r32[q] = v;
    e32[q] = 0.f;
    part = fma_rn(mul_rn(v, c32[q]), v, part);
  }
  const double s = block_sum<float>(part, red);
  if (threadIdx.x == 0) part_pt[ch] = s;
  const BatchProb P = pb[prob];
  if (last_block(cnt + prob, P.npc)) {
    const double rtz = block_sum_array(part_pt + P.pc0, P.npc, red);
    if (threadIdx.x == 0) {
      sc[prob].rtz1 = rtz;
      sc[prob].irtr0 = rtz;
      sc[prob].beta = 0.0;
      sc[prob].iactive = 1;
      sc[prob].pend = 0;
    }
  }
}

// x += |r| e for every active problem: the correction step of the FP64
// defect when the element operator is the fixed-point form (which takes x
// already corrected); the same fused multiply-add as the FP64-pipe forms'
// prologue.
__global__ void __launch_bounds__(kThreads)
    k_bxupd(double *__restrict__ x, const float *__restrict__ e, const long *__restrict__ pch_q0,
            const int *__restrict__ pch_prob, const BatchScalars *__restrict__ sc) {
  const int ch = blockIdx.x;
  const int prob = pch_prob[ch];
  if (!sc[prob].active) return;
  const double scale = sc[prob].rn;
  const long q0 = pch_q0[ch], q1 = pch_q0[ch + 1];
  for (long q = q0 + threadIdx.x; q < q1; q += kThreads)
    x[q] = fma_rn(scale, double(e[q]), x[q]);
}

// Initial state: x = 0, r = f, |f|_C; a problem with f = 0 (or no cycles
// allowed) is inactive from the start.
__global__ void __launch_bounds__(kThreads)
    k_binit(double *__restrict__ x, double *__restrict__ r, const double *__restrict__ f,
            const double *__restrict__ c, const long *__restrict__ pch_q0,
            const int *__restrict__ pch_prob, const BatchProb *__restrict__ pb,
            BatchScalars *sc, double *__restrict__ part_pt, unsigned *cnt, int max_outer) {
  __shared__ double red[32];
  const int ch = blockIdx.x;
  const int prob = pch_prob[ch];
  const long q0 = pch_q0[ch], q1 = pch_q0[ch + 1];
  double part = 0.0;
  for (long q = q0 + threadIdx.x; q < q1; q += kThreads) {
    const double fv = f[q];
    x[q] = 0.0;
    r[q] = fv;
    part = fma_rn(mul_rn(fv, c[q]), fv, part);
  }
  const double s = block_sum<double>(part, red);
  if (threadIdx.x == 0) part_pt[ch] = s;
  const BatchProb P = pb[prob];
  if (last_block(cnt + prob, P.npc)) {
    const double ff = block_sum_array(part_pt + P.pc0, P.npc, red);
    if (threadIdx.x == 0) {
      BatchScalars &S = sc[prob];
      S.rn0 = sqrt(ff);
      S.rn = S.rn0;
      S.rtr = ff;
      S.outer = 0;
      S.inner = 0;
      S.iactive = 0;
      S.active = (S.rn0 > 0.0 && max_outer > 0) ? 1 : 0;
    }
  }
}

// The loop condition: some problem still active and fewer than max_cycles
// cycles run (a bound that holds whatever the per-problem tests do).
__global__ void __launch_bounds__(kThreads)
    k_bcontrol(const BatchScalars *sc, int nprob, int *cycles, int reset, int max_cycles,
               cudaGraphConditionalHandle h) {
  int any = 0;
  for (int p = threadIdx.x; p < nprob; p += blockDim.x) any |= sc[p].active;
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) {
    const int cyc = reset ? 0 : *cycles + 1;
    *cycles = cyc;
    cudaGraphSetConditional(h, (any && cyc < max_cycles) ? 1u : 0u);
  }
}

// ---------------------------------------------------------- set-up kernels --
// setup_g (prox_setup.f:27-52) on one lx1 range
__global__ void k_bsetup_g(double *g, const double *wgt, int lx, long n) {
  const long l3 = long(lx) * lx * lx;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x) {
    const int rr = int(q % l3);
    const int i = rr % lx, j = (rr / lx) % lx, k = rr / (lx * lx);
    const double v = wgt[i] * wgt[j] * wgt[k];
    double *gp = g + 6 * q;
    gp[0] = v;
    gp[1] = 0.;
    gp[2] = 0.;
    gp[3] = v;
    gp[4] = 0.;
    gp[5] = v;
  }
}

// uniform [-1,1) per global point of one problem (its box numbering)
__global__ void k_brhs(double *f, int lx, int nelx, int nely, long n, uint64_t seed) {
  const long l3 = long(lx) * lx * lx;
  const int nn = lx - 1;
  const long ax = long(nn) * nelx + 1, ay = long(nn) * nely + 1;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x) {
    const long e = q / l3;
    const int rr = int(q % l3);
    const int i = rr % lx, j = (rr / lx) % lx, k = rr / (lx * lx);
    const long ex = e % nelx, ey = (e / nelx) % nely, ez = e / (long(nelx) * nely);
    const long id = 1 + (nn * ex + i) + (nn * ey + j) * ax + (nn * ez + k) * ax * ay;
    f[q] = uniform_pm1(seed, uint64_t(id));
  }
}

// multiplicity: c = 1 / group size on boundary groups (interior points keep 1)
__global__ void k_bmult(double *c, const int *off, const unsigned *idx, int ng) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int b = off[g], e = off[g + 1];
    const double v = 1.0 / double(e - b);
    for (int q = b; q < e; ++q) c[idx[q] & 0x7fffffffu] = v;
  }
}

// set_f's dssum, col2(c), mask (driver.f:88-101) on boundary groups
__global__ void k_bdssum_c_mask(double *f, const double *c, const int *off, const unsigned *idx,
                                int ng) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int b = off[g], e = off[g + 1];
    double t = f[idx[b] & 0x7fffffffu];
    for (int q = b + 1; q < e; ++q) t = add_rn(t, f[idx[q] & 0x7fffffffu]);
    for (int q = b; q < e; ++q) {
      const unsigned m = idx[q], id = m & 0x7fffffffu;
      f[id] = (m & 0x80000000u) ? 0.0 : mul_rn(t, c[id]);
    }
  }
}

__global__ void k_fill(double *a, double v, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = v;
}

template <typename T, typename S>
__global__ void k_conv(T *a, const S *b, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = T(b[q]);
}

__global__ void k_set_active(BatchScalars *sc, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nprob) {
    sc[p].active = 1;
    sc[p].iactive = 1;
    sc[p].rn = 1.0;
    sc[p].beta = 0.0;
  }
}

int grid_for(long n) {
  return int(std::max(1L, std::min<long>(152L * 8, (n + 255) / 256)));
}

// ------------------------------------------------------------- host set-up --
bool elem_boundary(int r, int lx) {
  const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
  return i == 0 || i == lx - 1 || j == 0 || j == lx - 1 || k == 0 || k == lx - 1;
}

// Element-boundary groups of one box problem in the order of the fused
// single-mesh pass: groups of points with one global id (set_vert_box), in
// ascending order of their first (smallest) local index, members ascending
// -- jl's local map order (gs.c:88-113, 330-357) -- plus every unshared
// boundary point as a group of one.  Members on a domain face carry bit 31.
void box_groups(int nelx, int nely, int nelz, int lx, std::vector<int> &off,
                std::vector<unsigned> &idx) {
  const int nelt = nelx * nely * nelz;
  const int l3 = lx * lx * lx;
  const long n = long(nelt) * l3;
  std::vector<int> lglel(nelt);
  for (int e = 0; e < nelt; ++e) lglel[e] = e + 1;
  std::vector<int64_t> glo(n);
  set_vert_box(glo.data(), lx, nelt, nelx, nely, lglel.data());
  std::vector<std::pair<int64_t, unsigned>> bp;
  bp.reserve(size_t(nelt) * (l3 - (lx > 2 ? (lx - 2) * (lx - 2) * (lx - 2) : 0)));
  for (long q = 0; q < n; ++q)
    if (elem_boundary(int(q % l3), lx)) bp.push_back({glo[q], unsigned(q)});
  std::sort(bp.begin(), bp.end());
  // runs of equal id; order runs by first member
  std::vector<std::pair<unsigned, std::pair<size_t, size_t>>> runs;
  for (size_t a = 0; a < bp.size();) {
    size_t b = a + 1;
    while (b < bp.size() && bp[b].first == bp[a].first) ++b;
    runs.push_back({bp[a].second, {a, b}});
    a = b;
  }
  std::sort(runs.begin(), runs.end());
  std::vector<unsigned char> face(nelt);
  for (int e = 0; e < nelt; ++e) face[e] = (unsigned char)face_bits(e + 1, nelx, nely, nelz);
  auto masked = [&](unsigned q) {
    const unsigned f = face[q / l3];
    if (!f) return false;
    const int rr = int(q % l3);
    const int i = rr % lx, j = (rr / lx) % lx, k = rr / (lx * lx);
    return ((f & 1u) && i == 0) || ((f & 2u) && i == lx - 1) || ((f & 4u) && j == 0) ||
           ((f & 8u) && j == lx - 1) || ((f & 16u) && k == 0) || ((f & 32u) && k == lx - 1);
  };
  off.clear();
  idx.clear();
  off.reserve(runs.size() + 1);
  idx.reserve(bp.size());
  for (const auto &rn : runs) {
    off.push_back(int(idx.size()));
    for (size_t q = rn.second.first; q < rn.second.second; ++q) {
      const unsigned m = bp[q].second;
      idx.push_back(m | (masked(m) ? 0x80000000u : 0u));
    }
  }
  off.push_back(int(idx.size()));
}

}  // namespace

// A batch of problems on the device.
struct Batch {
  struct Group {
    int lx = 0, el0 = 0, nel = 0;
    long pt0 = 0, n = 0;
    int pc0 = 0, npc = 0;     // its point chunks
    double *D64 = nullptr;
    float *D32 = nullptr;
    std::vector<double> EO;   // even-odd tables (host; empty for odd lx1)
    // the fixed-point FP64 operator's tables and converted metric for this
    // group's elements (even lx1)
    std::shared_ptr<Operator> fx;
    BatchTune tune;
  };
  int nprob = 0;
  std::vector<int> nelx, nely, nelz, lx;   // user order
  std::vector<int> slot;                   // user index -> internal index
  std::vector<BatchProb> P;                // internal order
  std::vector<int> P_user;                 // internal index -> user index
  std::vector<Group> groups;
  long n = 0;
  int nelt = 0, ng = 0, ngc = 0, npc = 0;
  // device
  double *x = nullptr, *f = nullptr, *g = nullptr, *c = nullptr, *r = nullptr, *w = nullptr;
  float *g32 = nullptr, *c32 = nullptr, *r32 = nullptr, *e32 = nullptr, *p32 = nullptr,
        *w32 = nullptr;
  float *p32b = nullptr;  // the inner CG's direction buffer of even iterations
  int *el_prob = nullptr, *off = nullptr, *gch_g0 = nullptr, *gch_prob = nullptr,
      *pch_prob = nullptr, *cycles = nullptr;
  unsigned *idx = nullptr, *cnt = nullptr;
  long *pch_q0 = nullptr;
  BatchProb *pb = nullptr;
  // c32 verified (at setup) as every problem's inverse multiplicity: the
  // elements' face bits, the extreme-index tables of each lx1, one flag
  unsigned char *cface = nullptr;
  unsigned *ext4 = nullptr;
  int *cf_flag = nullptr;
  bool cf_ok = false;
  BatchScalars *sc = nullptr;
  double *part_ax = nullptr, *part_gs = nullptr, *part_pt = nullptr;
  bool setup_done = false;
  // the solve graph
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double g_tol = -1.0, g_itol = -1.0;
  int g_inner = -1, g_outer = -1, g_wtest = -1, g_cf = -1, g_pair = -1;
  double itol = 0.0;  // 0: every cycle runs inner iterations; > 0: per-problem stop

  ~Batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (cap) cudaStreamDestroy(cap);
    for (auto &G : groups) {
      cudaFree(G.D64);
      cudaFree(G.D32);
    }
    void *ptrs[] = {x, f, g, c, r, w, g32, c32, r32, e32, p32, w32, el_prob, off, gch_g0,
                    gch_prob, pch_prob, cycles, idx, cnt, pch_q0, pb, sc, part_ax, part_gs,
                    part_pt, cface, ext4, cf_flag, p32b};
    for (void *p : ptrs)
      if (p) cudaFree(p);
  }

  // c formed in closed form by the inner iteration (verified at setup)
  bool closed_c() const { return cf_ok && g_mixed_closed_c; }
  // the inner CG's directions alternate between p32 (odd iterations) and
  // p32b (even), and x is updated once per pair (nb_set_paired_update)
  bool paired() const { return g_paired_update && p32b; }
  float *dir(int it) const { return paired() && !(it & 1) ? p32b : p32; }
  float *dir_old(int it) const { return paired() && (it & 1) ? p32b : p32; }
  int launch_inner_ax(int it, cudaStream_t s) const {
    for (const auto &G : groups) {
      BaxArgs<float> a{};
      a.w = w32;
      a.u = r32;
      a.p = dir(it);
      a.pold = dir_old(it);
      a.g = g32;
      a.c = c32;
      a.c_unit_interior = closed_c() ? 1 : 0;
      a.D = G.D32;
      a.eo_h = G.EO.empty() ? nullptr : G.EO.data();
      a.el_prob = el_prob;
      a.sc = sc;
      a.partial = part_ax;
      a.pt0 = G.pt0;
      a.el0 = G.el0;
      a.nel = G.nel;
      a.first = it == 1;
      a.err = device_error_word();
      a.wait_test = wait_test_mode();
      NB_TRY(batch_ax_f32(G.lx, G.tune.epb32, G.tune.rd32, a, s));
    }
    return NB_OK;
  }
  // The FP64 defect's element operator for one group in shape epb64
  // (kFxShape: the fixed-point form after a separate x += |r| e).
  int defect_group_ax(const Group &G, int epb64, cudaStream_t s) const {
    if (epb64 == kFxShape) {
      if (!G.fx) return fail(NB_ERR_UNSUPPORTED, "batched solve: no fixed-point form for lx1=%d",
                             G.lx);
      k_bxupd<<<G.npc, kThreads, 0, s>>>(x, e32, pch_q0 + G.pc0, pch_prob + G.pc0, sc);
      NB_CUDA(cudaGetLastError());
      AxArgs<double> a{};
      a.w = w + G.pt0;
      a.p = x + G.pt0;
      a.c = c + G.pt0;
      a.f = f + G.pt0;
      a.r = r + G.pt0;
      a.partial = part_ax + G.el0;
      a.nelt = G.nel;
      a.gfx = G.fx->gfx;
      a.gexp = G.fx->gexp;
      a.el_prob = el_prob + G.el0;
      a.act = &sc[0].active;
      a.act_stride = int(sizeof(BatchScalars) / sizeof(int));
      a.err = device_error_word();
      return launch_ax_fx_m2(*G.fx, a, s);
    }
    BaxArgs<double> a{};
    a.w = w;
    a.p = x;
    a.g = g;
    a.c = c;
    a.D = G.D64;
    a.eo_h = G.EO.empty() ? nullptr : G.EO.data();
    a.f = f;
    a.r = r;
    a.e = e32;
    a.el_prob = el_prob;
    a.sc = sc;
    a.partial = part_ax;
    a.pt0 = G.pt0;
    a.el0 = G.el0;
    a.nel = G.nel;
    a.err = device_error_word();
    a.wait_test = wait_test_mode();
    return batch_ax_f64(G.lx, epb64, a, s);
  }
  // the fixed-point metric of every group that uses the fixed-point form
  int convert_metric(cudaStream_t s) const {
    for (const auto &G : groups)
      if (G.fx && G.tune.epb64 == kFxShape) {
        metric_fx_invalidate(*G.fx);
        NB_TRY(metric_fx_prepare(*G.fx, g + 6 * G.pt0, s));
      }
    return NB_OK;
  }
  int launch_defect_ax(cudaStream_t s) const {
    for (const auto &G : groups) NB_TRY(defect_group_ax(G, G.tune.epb64, s));
    return NB_OK;
  }
  static int batch_ax_f32(int lx, int epb, int rd, BaxArgs<float> a, cudaStream_t s) {
    if (!a.pold) a.pold = a.p;  // MODE 1 reads the old direction from pold
    switch (lx) {
      case 4: return batch_ax_f32_lx<4>(epb, rd, a, s);
      case 6: return batch_ax_f32_lx<6>(epb, rd, a, s);
      case 8: return batch_ax_f32_lx<8>(epb, rd, a, s);
      case 10: return batch_ax_f32_lx<10>(epb, rd, a, s);
      case 12: return batch_ax_f32_lx<12>(epb, rd, a, s);
    }
    return fail(NB_ERR_UNSUPPORTED, "batched solve: lx1=%d not supported", lx);
  }
  static int batch_ax_f64(int lx, int epb, const BaxArgs<double> &a, cudaStream_t s) {
    switch (lx) {
      case 4: return batch_ax_f64_lx<4>(epb, a, s);
      case 6: return batch_ax_f64_lx<6>(epb, a, s);
      case 8: return batch_ax_f64_lx<8>(epb, a, s);
      case 10: return batch_ax_f64_lx<10>(epb, a, s);
      case 12: return batch_ax_f64_lx<12>(epb, a, s);
    }
    return fail(NB_ERR_UNSUPPORTED, "batched solve: lx1=%d not supported", lx);
  }

  // Records phase mark e on s (a no-op without one); under stream capture
  // the record becomes an event node of the graph.
  static int mark(const cudaEvent_t *e, cudaStream_t s) {
    if (e) NB_CUDA(cudaEventRecordWithFlags(*e, s, cudaEventRecordExternal));
    return NB_OK;
  }

  // one inner FP32 iteration / the FP64 defect, for all active problems;
  // with mk, an event after each of the iteration's three (the defect's
  // two) launches
  int inner_iteration(int it, int max_inner, cudaStream_t s,
                      const cudaEvent_t *mk = nullptr) const {
    NB_TRY(launch_inner_ax(it, s));
    NB_TRY(mark(mk, s));
    float *pc = dir(it);
    k_bgs_fin<<<ngc, kThreads, 0, s>>>(w32, pc, c32, off, idx, gch_g0, gch_prob, pb, sc, part_gs,
                                       part_ax, cnt);
    NB_CUDA(cudaGetLastError());
    NB_TRY(mark(mk ? mk + 1 : nullptr, s));
    const unsigned char *cf = closed_c() ? cface : nullptr;
    if (paired() && (it & 1) && it < max_inner)
      k_bupd<1><<<npc, kThreads, 0, s>>>(e32, r32, pc, w32, c32, pch_q0, pch_prob, pb, sc,
                                         part_pt, cnt + nprob, it, max_inner, itol, cf, ext4,
                                         nullptr);
    else if (paired() && !(it & 1))
      k_bupd<2><<<npc, kThreads, 0, s>>>(e32, r32, pc, w32, c32, pch_q0, pch_prob, pb, sc,
                                         part_pt, cnt + nprob, it, max_inner, itol, cf, ext4,
                                         dir_old(it));
    else
      k_bupd<0><<<npc, kThreads, 0, s>>>(e32, r32, pc, w32, c32, pch_q0, pch_prob, pb, sc,
                                         part_pt, cnt + nprob, it, max_inner, itol, cf, ext4,
                                         nullptr);
    NB_CUDA(cudaGetLastError());
    NB_TRY(mark(mk ? mk + 2 : nullptr, s));
    return NB_OK;
  }
  int defect(double tol, int max_outer, cudaStream_t s, const cudaEvent_t *mk = nullptr) const {
    if (paired()) {  // the x updates deferred by inner CGs that stopped mid-pair
      k_bflush<<<npc, kThreads, 0, s>>>(e32, p32, pch_q0, pch_prob, sc);
      NB_CUDA(cudaGetLastError());
    }
    NB_TRY(launch_defect_ax(s));
    NB_TRY(mark(mk, s));
    k_bgs_res<<<ngc, kThreads, 0, s>>>(w, x, f, r, c, off, idx, gch_g0, gch_prob, pb, sc, part_gs,
                                       part_ax, cnt + 2 * nprob, tol, max_outer);
    NB_CUDA(cudaGetLastError());
    NB_TRY(mark(mk ? mk + 1 : nullptr, s));
    return NB_OK;
  }
  int scale(cudaStream_t s) const {
    k_bscale<<<npc, kThreads, 0, s>>>(r32, e32, r, c32, pch_q0, pch_prob, pb, sc, part_pt,
                                      cnt + 3 * nprob);
    NB_CUDA(cudaGetLastError());
    return NB_OK;
  }
  // initial norms, and the fixed-point metric of the solve (g may have
  // changed since the last one)
  int init(int max_outer, cudaStream_t s) const {
    NB_TRY(convert_metric(s));
    k_binit<<<npc, kThreads, 0, s>>>(x, r, f, c, pch_q0, pch_prob, pb, sc, part_pt,
                                     cnt + 3 * nprob, max_outer);
    NB_CUDA(cudaGetLastError());
    return NB_OK;
  }

  // The solve of build_graph launched one cycle at a time: each cycle is a
  // graph of the same kernels with an event after every launch, and the
  // loop condition (some problem active, fewer than max_outer + 1 cycles)
  // is read on the host between cycles.  Adds each phase's device time
  // (kBatchPhases entries, nb_batch_time_phases's order) to ms.
  static constexpr int kBatchPhases = 7;
  int timed_solve(double tol, int inner, int max_outer, cudaStream_t s, double *ms,
                  int *ncyc) {
    struct Owned {
      std::vector<cudaEvent_t> ev;
      cudaGraph_t g = nullptr;
      cudaGraphExec_t x = nullptr;
      ~Owned() {
        if (x) cudaGraphExecDestroy(x);
        if (g) cudaGraphDestroy(g);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
      }
    } o;
    // events: start, after scale, 3 per inner iteration, 2 for the defect
    const int nev = 3 * inner + 4;
    std::vector<int> phase(nev, -1);   // phase of the interval ending at event q
    phase[1] = 1;
    for (int it = 0; it < inner; ++it)
      for (int k = 0; k < 3; ++k) phase[2 + 3 * it + k] = 2 + k;
    phase[nev - 2] = 5;
    phase[nev - 1] = 6;
    for (int q = 0; q < nev; ++q) {
      cudaEvent_t e;
      NB_CUDA(cudaEventCreate(&e));
      o.ev.push_back(e);
    }
    if (!cap) NB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    NB_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed));
    int st = mark(&o.ev[0], cap);
    if (!st) st = scale(cap);
    if (!st) st = mark(&o.ev[1], cap);
    for (int it = 1; it <= inner && !st; ++it)
      st = inner_iteration(it, inner, cap, &o.ev[2 + 3 * (it - 1)]);
    if (!st) st = defect(tol, max_outer, cap, &o.ev[nev - 2]);
    const cudaError_t ce = cudaStreamEndCapture(cap, &o.g);
    if (st) return st;
    if (ce != cudaSuccess)
      return fail(NB_ERR_CUDA, "batched phase timing: capture: %s", cudaGetErrorString(ce));
    NB_CUDA(cudaGraphInstantiate(&o.x, o.g, 0));
    cudaEvent_t i0 = o.ev[0], i1 = o.ev[1];
    NB_CUDA(cudaEventRecord(i0, s));
    NB_TRY(init(max_outer, s));
    NB_CUDA(cudaEventRecord(i1, s));
    NB_CUDA(cudaEventSynchronize(i1));
    float t = 0.f;
    NB_CUDA(cudaEventElapsedTime(&t, i0, i1));
    ms[0] += t;
    std::vector<BatchScalars> h(nprob);
    const int max_cycles = max_outer + 1;
    int cyc = 0;
    for (;;) {
      NB_CUDA(cudaMemcpyAsync(h.data(), sc, nprob * sizeof(BatchScalars),
                              cudaMemcpyDeviceToHost, s));
      NB_CUDA(cudaStreamSynchronize(s));
      int any = 0;
      for (const BatchScalars &q : h) any |= q.active;
      if (!any || cyc >= max_cycles) break;
      NB_CUDA(cudaGraphLaunch(o.x, s));
      NB_CUDA(cudaEventSynchronize(o.ev[nev - 1]));
      for (int q = 1; q < nev; ++q) {
        NB_CUDA(cudaEventElapsedTime(&t, o.ev[q - 1], o.ev[q]));
        ms[phase[q]] += t;
      }
      ++cyc;
    }
    NB_CUDA(cudaMemcpyAsync(cycles, &cyc, sizeof(int), cudaMemcpyHostToDevice, s));
    NB_CUDA(cudaStreamSynchronize(s));
    NB_TRY(device_error_check(s));
    *ncyc = cyc;
    return NB_OK;
  }

  int build_graph(double tol, int inner, int max_outer) {
    if (exec && tol == g_tol && inner == g_inner && max_outer == g_outer && itol == g_itol &&
        wait_test_mode() == g_wtest && int(closed_c()) == g_cf && int(paired()) == g_pair)
      return NB_OK;
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    if (!cap) NB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t G = nullptr;
    NB_CUDA(cudaGraphCreate(&G, 0));
    graph = G;
    cudaGraphConditionalHandle h;
    NB_CUDA(cudaGraphConditionalHandleCreate(&h, G, 0, 0));
    const int max_cycles = max_outer + 1;
    // initial norms, then the first value of the loop condition, captured
    // into the graph itself (the node setting the condition must belong to
    // the graph that owns the handle)
    NB_CUDA(cudaStreamBeginCaptureToGraph(cap, G, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed));
    {
      const int st0 = init(max_outer, cap);
      k_bcontrol<<<1, kThreads, 0, cap>>>(sc, nprob, cycles, 1, max_cycles, h);
      cudaGraph_t got = nullptr;
      NB_CUDA(cudaStreamEndCapture(cap, &got));
      NB_TRY(st0);
    }
    // the loop follows the capture's last node (the one without dependents)
    size_t nn = 0;
    NB_CUDA(cudaGraphGetNodes(G, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    NB_CUDA(cudaGraphGetNodes(G, nodes.data(), &nn));
    cudaGraphNode_t ninit = nullptr;
    int nlast = 0;
    for (cudaGraphNode_t q : nodes) {
      size_t nd = 0;
      NB_CUDA(cudaGraphNodeGetDependentNodes(q, nullptr, nullptr, &nd));
      if (nd == 0) {
        ninit = q;
        ++nlast;
      }
    }
    if (nlast != 1) return fail(NB_ERR_CUDA, "batched solve: unexpected initial graph");
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t nloop;
    NB_CUDA(cudaGraphAddNode(&nloop, G, &ninit, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    // one cycle: scale, inner CG, FP64 defect, loop condition
    NB_CUDA(cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed));
    int st = scale(cap);
    for (int it = 1; it <= inner && !st; ++it) st = inner_iteration(it, inner, cap);
    if (!st) st = defect(tol, max_outer, cap);
    if (!st) {
      k_bcontrol<<<1, kThreads, 0, cap>>>(sc, nprob, cycles, 0, max_cycles, h);
      if (cudaGetLastError() != cudaSuccess) st = fail(NB_ERR_CUDA, "batched solve: capture");
    }
    cudaGraph_t got = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cap, &got);
    if (st) return st;
    if (ce != cudaSuccess) return fail(NB_ERR_CUDA, "batched solve: capture: %s",
                                       cudaGetErrorString(ce));
    NB_CUDA(cudaGraphInstantiate(&exec, G, 0));
    g_tol = tol;
    g_inner = inner;
    g_outer = max_outer;
    g_itol = itol;
    g_wtest = wait_test_mode();
    g_cf = int(closed_c());
    g_pair = int(paired());
    return NB_OK;
  }
};

namespace {

template <typename T>
int dalloc(T **p, size_t count) {
  if (count == 0) count = 1;
  if (cudaMalloc(p, count * sizeof(T)) != cudaSuccess)
    return fail(NB_ERR_CUDA, "batched solve: out of device memory (%zu bytes)",
                count * sizeof(T));
  return NB_OK;
}

template <typename T>
int upload(T **p, const std::vector<T> &h) {
  NB_TRY(dalloc(p, h.size()));
  if (!h.empty())
    NB_CUDA(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return NB_OK;
}

int batch_build(Batch *B, int nprob, const int *nx, const int *ny, const int *nz,
                const int *lx) {
  B->nprob = nprob;
  B->nelx.assign(nx, nx + nprob);
  B->nely.assign(ny, ny + nprob);
  B->nelz.assign(nz, nz + nprob);
  B->lx.assign(lx, lx + nprob);
  for (int p = 0; p < nprob; ++p) {
    if (nx[p] <= 0 || ny[p] <= 0 || nz[p] <= 0)
      return fail(NB_ERR_ARG, "batched solve: problem %d box %dx%dx%d", p, nx[p], ny[p], nz[p]);
    if (!(lx[p] == 4 || lx[p] == 6 || lx[p] == 8 || lx[p] == 10 || lx[p] == 12))
      return fail(NB_ERR_UNSUPPORTED, "batched solve: problem %d lx1=%d (supported 4,6,8,10,12)",
                  p, lx[p]);
  }
  // internal order: by lx1, then by user index
  std::vector<int> order(nprob);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return lx[a] < lx[b]; });
  B->slot.assign(nprob, 0);
  B->P_user = order;
  for (int s = 0; s < nprob; ++s) B->slot[order[s]] = s;
  // per-problem groups (host), built in parallel
  std::vector<std::vector<int>> offs(nprob);
  std::vector<std::vector<unsigned>> idxs(nprob);
  {
    const int nth = std::max(1, std::min<int>(nprob, int(std::thread::hardware_concurrency())));
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t)
      th.emplace_back([&, t]() {
        for (int s = t; s < nprob; s += nth) {
          const int p = order[s];
          box_groups(nx[p], ny[p], nz[p], lx[p], offs[s], idxs[s]);
        }
      });
    for (auto &t : th) t.join();
  }
  // concatenation
  B->P.resize(nprob);
  std::vector<int> el_prob, off_all, gch_g0, gch_prob, pch_prob;
  std::vector<unsigned> idx_all, ext_all;
  std::vector<long> pch_q0;
  long pt = 0;
  int el = 0, gbase = 0, ext_lx0 = 0;
  for (int s = 0; s < nprob; ++s) {
    const int p = order[s];
    const long l3 = long(lx[p]) * lx[p] * lx[p];
    const long nelt = long(nx[p]) * ny[p] * nz[p];
    if (pt + nelt * l3 >= (1L << 31) || el + nelt >= (1L << 31))
      return fail(NB_ERR_UNSUPPORTED, "batched solve: more than 2^31-1 points in the batch");
    BatchProb &Q = B->P[s];
    Q.pt0 = pt;
    Q.n = nelt * l3;
    Q.el0 = el;
    Q.nelt = int(nelt);
    Q.lx = lx[p];
    if (s == 0 || lx[order[s - 1]] != lx[p]) {  // problems are sorted by lx1
      ext_lx0 = int(ext_all.size());
      const std::vector<unsigned> t = ext_table(lx[p]);
      ext_all.insert(ext_all.end(), t.begin(), t.end());
    }
    Q.ext0 = ext_lx0;
    for (long e = 0; e < nelt; ++e) el_prob.push_back(s);
    const int ngp = int(offs[s].size()) - 1;
    for (int q = 0; q < ngp; ++q)
      if (offs[s][q + 1] - offs[s][q] > 8)
        return fail(NB_ERR_STATE, "batched solve: a boundary group of more than 8 points");
    for (int q = 0; q < ngp; ++q) off_all.push_back(offs[s][q] + int(idx_all.size()));
    for (unsigned m : idxs[s])
      idx_all.push_back(unsigned(pt + (m & 0x7fffffffu)) | (m & 0x80000000u));
    Q.gc0 = int(gch_prob.size());
    for (int a = 0; a < ngp; a += kGroupChunk) {
      gch_g0.push_back(gbase + a);
      gch_prob.push_back(s);
    }
    Q.ngc = int(gch_prob.size()) - Q.gc0;
    Q.pc0 = int(pch_prob.size());
    for (long a = 0; a < Q.n; a += kPointChunk) {
      pch_q0.push_back(pt + a);
      pch_prob.push_back(s);
    }
    Q.npc = int(pch_prob.size()) - Q.pc0;
    gbase += ngp;
    pt += Q.n;
    el += int(nelt);
    if (B->groups.empty() || B->groups.back().lx != lx[p]) {
      Batch::Group G;
      G.lx = lx[p];
      G.el0 = Q.el0;
      G.pt0 = Q.pt0;
      G.pc0 = Q.pc0;
      B->groups.push_back(G);
    }
    B->groups.back().nel += int(nelt);
    B->groups.back().n += Q.n;
    B->groups.back().npc += Q.npc;
  }
  off_all.push_back(int(idx_all.size()));
  gch_g0.push_back(gbase);
  pch_q0.push_back(pt);
  B->n = pt;
  B->nelt = el;
  B->ng = gbase;
  B->ngc = int(gch_prob.size());
  B->npc = int(pch_prob.size());
  const long n = B->n;
  NB_TRY(dalloc(&B->x, n));
  NB_TRY(dalloc(&B->f, n));
  NB_TRY(dalloc(&B->g, 6 * n));
  NB_TRY(dalloc(&B->c, n));
  NB_TRY(dalloc(&B->r, n));
  NB_TRY(dalloc(&B->w, n));
  NB_TRY(dalloc(&B->g32, 6 * n));
  NB_TRY(dalloc(&B->c32, n));
  NB_TRY(dalloc(&B->r32, n));
  NB_TRY(dalloc(&B->e32, n));
  NB_TRY(dalloc(&B->p32, n));
  NB_TRY(dalloc(&B->p32b, n));
  NB_CUDA(cudaMemset(B->p32b, 0, n * sizeof(float)));
  NB_TRY(dalloc(&B->w32, n));
  NB_TRY(upload(&B->el_prob, el_prob));
  NB_TRY(upload(&B->off, off_all));
  NB_TRY(upload(&B->idx, idx_all));
  NB_TRY(upload(&B->gch_g0, gch_g0));
  NB_TRY(upload(&B->gch_prob, gch_prob));
  NB_TRY(upload(&B->pch_q0, pch_q0));
  NB_TRY(upload(&B->pch_prob, pch_prob));
  NB_TRY(upload(&B->pb, B->P));
  NB_TRY(upload(&B->ext4, ext_all));
  NB_TRY(dalloc(&B->cface, size_t(B->nelt)));
  NB_TRY(dalloc(&B->cf_flag, 1));
  NB_TRY(dalloc(&B->sc, nprob));
  NB_TRY(dalloc(&B->cnt, 4 * size_t(nprob)));
  NB_TRY(dalloc(&B->cycles, 1));
  NB_TRY(dalloc(&B->part_ax, B->nelt));
  NB_TRY(dalloc(&B->part_gs, B->ngc));
  NB_TRY(dalloc(&B->part_pt, B->npc));
  NB_CUDA(cudaMemset(B->cnt, 0, 4 * size_t(nprob) * sizeof(unsigned)));
  NB_CUDA(cudaMemset(B->sc, 0, nprob * sizeof(BatchScalars)));
  for (auto &G : B->groups) {
    const int L = G.lx;
    std::vector<double> a(L * L), b(L), cc(L * L), d(L * L), zz(L);
    semhat(a.data(), b.data(), cc.data(), d.data(), zz.data(), L - 1);
    std::vector<float> d32(d.begin(), d.end());
    NB_TRY(upload(&G.D64, d));
    NB_TRY(upload(&G.D32, d32));
    if (!even_odd_tables(d, L, G.EO)) G.EO.clear();
    auto op = std::make_shared<Operator>();
    op->lx = L;
    op->n = G.n;
    op->nelt = G.nel;
    op->fx_ok = fx_tables(d, L, op->FXhi, op->FXlo, &op->fx_fc);
    if (op->fx_ok) G.fx = op;
    // default shape: the first listed (the even-odd form where lx1 is even)
    const auto s32 = batch_shapes_f32(L);
    const auto s64 = batch_shapes_f64(L);
    G.tune.epb32 = s32.front().first;
    G.tune.rd32 = s32.front().second;
    G.tune.epb64 = s64.front();
  }
  return NB_OK;
}

}  // namespace

std::vector<std::pair<int, int>> batch_shapes_f32(int lx) {
  std::vector<int> e;
  switch (lx) {
    case 4: e = {4, 8, 16}; break;
    case 6: e = {2, 4, 8}; break;
    default: e = {1, 2, 4}; break;
  }
  // the even-odd form first (even lx1), then register D, then shared D,
  // smallest element count first
  std::vector<std::pair<int, int>> out;
  if (lx % 2 == 0) out.push_back({1, 2});
  for (int rd = 1; rd >= 0; --rd)
    for (int v : e) out.push_back({v, rd});
  return out;
}

std::vector<int> batch_shapes_f64(int lx) {
  std::vector<int> out;
  if (lx % 2 == 0) out.push_back(kFxShape);   // fixed point on the integer pipes
  if (lx % 2 == 0) out.push_back(0);          // even-odd form on the FP64 pipe
  switch (lx) {
    case 4: out.insert(out.end(), {4, 8}); break;
    case 6: out.insert(out.end(), {2, 4}); break;
    default: out.insert(out.end(), {1, 2}); break;
  }
  return out;
}

}  // namespace nb

using namespace nb;

struct nb_batch {
  Batch B;
};

extern "C" {

int nb_batch_create(nb_batch **out, int nprob, const int *nelx, const int *nely,
                    const int *nelz, const int *lx1) {
  clear_status();
  if (!out) return fail(NB_ERR_ARG, "nb_batch_create: null output");
  *out = nullptr;
  if (nprob <= 0 || !nelx || !nely || !nelz || !lx1)
    return fail(NB_ERR_ARG, "nb_batch_create: %d problems", nprob);
  nb_batch *b = new nb_batch();
  const int st = batch_build(&b->B, nprob, nelx, nely, nelz, lx1);
  if (st) {
    delete b;
    return st;
  }
  *out = b;
  return NB_OK;
}

int nb_batch_destroy(nb_batch *b) {
  clear_status();
  if (!b) return NB_OK;
  cudaStreamSynchronize(lib_stream());
  delete b;
  return NB_OK;
}

int nb_batch_info(const nb_batch *b, long *npts, int *nelt, int *nlx) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  if (npts) *npts = b->B.n;
  if (nelt) *nelt = b->B.nelt;
  if (nlx) *nlx = int(b->B.groups.size());
  return NB_OK;
}

int nb_batch_problem(const nb_batch *b, int prob, long *pt_offset, long *npts, int *lx1) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  if (prob < 0 || prob >= b->B.nprob) return fail(NB_ERR_ARG, "problem %d out of range", prob);
  const BatchProb &Q = b->B.P[b->B.slot[prob]];
  if (pt_offset) *pt_offset = Q.pt0;
  if (npts) *npts = Q.n;
  if (lx1) *lx1 = b->B.lx[prob];
  return NB_OK;
}

int nb_batch_arrays(nb_batch *b, double **x, double **f, double **g, double **c) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  if (x) *x = b->B.x;
  if (f) *f = b->B.f;
  if (g) *g = b->B.g;
  if (c) *c = b->B.c;
  return NB_OK;
}

int nb_batch_setup(nb_batch *b, uint64_t seed) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  Batch &B = b->B;
  cudaStream_t s = lib_stream();
  for (auto &G : B.groups) {
    const int L = G.lx;
    std::vector<double> a(L * L), wb(L), cc(L * L), d(L * L), zz(L);
    semhat(a.data(), wb.data(), cc.data(), d.data(), zz.data(), L - 1);
    double *dw = nullptr;
    NB_TRY(upload(&dw, wb));
    k_bsetup_g<<<grid_for(G.n), 256, 0, s>>>(B.g + 6 * G.pt0, dw, L, G.n);
    const cudaError_t e = cudaGetLastError();
    NB_CUDA(cudaStreamSynchronize(s));
    cudaFree(dw);
    if (e != cudaSuccess) return fail(NB_ERR_CUDA, "nb_batch_setup: %s", cudaGetErrorString(e));
  }
  k_fill<<<grid_for(B.n), 256, 0, s>>>(B.c, 1.0, B.n);
  k_bmult<<<grid_for(B.ng), 256, 0, s>>>(B.c, B.off, B.idx, B.ng);
  for (int p = 0; p < B.nprob; ++p) {
    const BatchProb &Q = B.P[B.slot[p]];
    k_brhs<<<grid_for(Q.n), 256, 0, s>>>(B.f + Q.pt0, B.lx[p], B.nelx[p], B.nely[p], Q.n,
                                         seed + uint64_t(p));
  }
  k_bdssum_c_mask<<<grid_for(B.ng), 256, 0, s>>>(B.f, B.c, B.off, B.idx, B.ng);
  k_conv<float, double><<<grid_for(6 * B.n), 256, 0, s>>>(B.g32, B.g, 6 * B.n);
  k_conv<float, double><<<grid_for(B.n), 256, 0, s>>>(B.c32, B.c, B.n);
  NB_CUDA(cudaGetLastError());
  // whether c32 is every problem's inverse multiplicity in closed form
  NB_CUDA(cudaMemsetAsync(B.cf_flag, 0xFF, sizeof(int), s));
  k_bc_closed_form<<<std::max(1, std::min(B.nelt, grid_for(long(B.nelt) * 256))), 256, 0, s>>>(
      B.c32, B.el_prob, B.pb, B.nelt, B.cface, B.cf_flag);
  NB_CUDA(cudaGetLastError());
  int cf_h = 0;
  NB_CUDA(cudaMemcpyAsync(&cf_h, B.cf_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  // the fixed-point metric (allocated here, outside any graph capture;
  // every solve converts it again)
  for (auto &G : B.groups)
    if (G.fx) {
      metric_fx_invalidate(*G.fx);
      NB_TRY(metric_fx_prepare(*G.fx, B.g + 6 * G.pt0, s));
    }
  NB_CUDA(cudaStreamSynchronize(s));
  B.cf_ok = cf_h != 0;
  B.setup_done = true;
  return NB_OK;
}

int nb_batch_set_tuning(nb_batch *b, int lx1, int epb32, int rd32, int epb64) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  for (auto &G : b->B.groups)
    if (G.lx == lx1) {
      bool ok32 = false, ok64 = false;
      for (auto sh : batch_shapes_f32(lx1)) ok32 |= sh.first == epb32 && sh.second == rd32;
      for (int v : batch_shapes_f64(lx1)) ok64 |= v == epb64;
      if (!ok32 || !ok64)
        return fail(NB_ERR_UNSUPPORTED, "nb_batch_set_tuning: shape not instantiated for lx1=%d",
                    lx1);
      G.tune.epb32 = epb32;
      G.tune.rd32 = rd32;
      G.tune.epb64 = epb64;
      if (b->B.exec) {
        cudaGraphExecDestroy(b->B.exec);
        b->B.exec = nullptr;
      }
      return NB_OK;
    }
  return fail(NB_ERR_ARG, "nb_batch_set_tuning: no problem with lx1=%d", lx1);
}

int nb_batch_get_tuning(const nb_batch *b, int lx1, int *epb32, int *rd32, int *epb64,
                        float *ms32, float *ms64) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  for (const auto &G : b->B.groups)
    if (G.lx == lx1) {
      if (epb32) *epb32 = G.tune.epb32;
      if (rd32) *rd32 = G.tune.rd32;
      if (epb64) *epb64 = G.tune.epb64;
      if (ms32) *ms32 = G.tune.ms32;
      if (ms64) *ms64 = G.tune.ms64;
      return NB_OK;
    }
  return fail(NB_ERR_ARG, "nb_batch_get_tuning: no problem with lx1=%d", lx1);
}

// The autotuner: every instantiated shape of the FP32 inner operator and of
// the FP64 defect operator is timed on the batch's own elements of each
// lx1 (CUDA events, reps launches after one warm-up), the fastest kept.
int nb_batch_tune(nb_batch *b, int reps) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  Batch &B = b->B;
  if (!B.setup_done) return fail(NB_ERR_STATE, "nb_batch_tune: call nb_batch_setup first");
  if (reps < 1) reps = 1;
  cudaStream_t s = lib_stream();
  // scratch state: every problem active, inputs zeroed
  NB_CUDA(cudaMemsetAsync(B.p32, 0, B.n * sizeof(float), s));
  NB_CUDA(cudaMemsetAsync(B.r32, 0, B.n * sizeof(float), s));
  NB_CUDA(cudaMemsetAsync(B.e32, 0, B.n * sizeof(float), s));
  NB_CUDA(cudaMemsetAsync(B.x, 0, B.n * sizeof(double), s));
  k_set_active<<<(B.nprob + 255) / 256, 256, 0, s>>>(B.sc, B.nprob);
  NB_CUDA(cudaGetLastError());
  cudaEvent_t e0, e1;
  NB_CUDA(cudaEventCreate(&e0));
  NB_CUDA(cudaEventCreate(&e1));
  int st = NB_OK;
  for (auto &G : B.groups) {
    float best = 1e30f;
    BatchTune t = G.tune;
    for (auto sh : batch_shapes_f32(G.lx)) {
      BaxArgs<float> a{};
      a.w = B.w32;
      a.u = B.r32;
      a.p = B.p32;
      a.g = B.g32;
      a.c = B.c32;
      a.D = G.D32;
      a.eo_h = G.EO.empty() ? nullptr : G.EO.data();
      a.el_prob = B.el_prob;
      a.sc = B.sc;
      a.partial = B.part_ax;
      a.pt0 = G.pt0;
      a.el0 = G.el0;
      a.nel = G.nel;
      a.first = 0;
      a.err = device_error_word();
      a.wait_test = wait_test_mode();
      st = Batch::batch_ax_f32(G.lx, sh.first, sh.second, a, s);
      if (st) break;
      cudaEventRecord(e0, s);
      for (int q = 0; q < reps; ++q) Batch::batch_ax_f32(G.lx, sh.first, sh.second, a, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= reps;
      if (ms < best) {
        best = ms;
        t.epb32 = sh.first;
        t.rd32 = sh.second;
        t.ms32 = ms;
      }
    }
    if (st) break;
    best = 1e30f;
    for (int epb : batch_shapes_f64(G.lx)) {
      st = B.defect_group_ax(G, epb, s);
      if (st) break;
      cudaEventRecord(e0, s);
      for (int q = 0; q < reps; ++q) B.defect_group_ax(G, epb, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= reps;
      if (ms < best) {
        best = ms;
        t.epb64 = epb;
        t.ms64 = ms;
      }
    }
    if (st) break;
    G.tune = t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  NB_CUDA(cudaStreamSynchronize(s));
  NB_CUDA(cudaGetLastError());
  if (B.exec) {
    cudaGraphExecDestroy(B.exec);
    B.exec = nullptr;
  }
  return NB_OK;
}

// Enqueues the whole solve (one graph launch) on the library stream.
int nb_batch_set_inner_tol(nb_batch *b, double itol) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  if (!(itol >= 0.0 && itol < 1.0)) return fail(NB_ERR_ARG, "inner tolerance %g", itol);
  b->B.itol = itol;
  return NB_OK;
}

int nb_batch_solve(nb_batch *b, double tol, int inner_iters, int max_outer) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  Batch &B = b->B;
  if (!B.setup_done) return fail(NB_ERR_STATE, "nb_batch_solve: call nb_batch_setup first");
  if (inner_iters < 1 || max_outer < 0 || !(tol >= 0.0))
    return fail(NB_ERR_ARG, "nb_batch_solve: inner_iters=%d max_outer=%d", inner_iters,
                max_outer);
  NB_TRY(B.build_graph(tol, inner_iters, max_outer));
  NB_CUDA(cudaGraphLaunch(B.exec, lib_stream()));
  return NB_OK;
}

int nb_batch_time_phases(nb_batch *b, double tol, int inner_iters, int max_outer, double *ms,
                         int *cycles) {
  clear_status();
  if (!b || !ms) return fail(NB_ERR_ARG, "nb_batch_time_phases: null argument");
  Batch &B = b->B;
  if (!B.setup_done) return fail(NB_ERR_STATE, "nb_batch_time_phases: call nb_batch_setup first");
  if (inner_iters < 1 || max_outer < 0 || !(tol >= 0.0))
    return fail(NB_ERR_ARG, "nb_batch_time_phases: inner_iters=%d max_outer=%d", inner_iters,
                max_outer);
  for (int k = 0; k < Batch::kBatchPhases; ++k) ms[k] = 0.0;
  int cyc = 0;
  NB_TRY(B.timed_solve(tol, inner_iters, max_outer, lib_stream(), ms, &cyc));
  if (cycles) *cycles = cyc;
  return NB_OK;
}

int nb_batch_result(const nb_batch *b, int prob, int *outer, int *inner, double *relres) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  if (prob < 0 || prob >= b->B.nprob) return fail(NB_ERR_ARG, "problem %d out of range", prob);
  BatchScalars S;
  cudaStream_t s = lib_stream();
  NB_CUDA(cudaMemcpyAsync(&S, b->B.sc + b->B.slot[prob], sizeof(S), cudaMemcpyDeviceToHost, s));
  NB_TRY(device_error_check(s));
  if (outer) *outer = S.outer;
  if (inner) *inner = S.inner;
  if (relres) *relres = S.rn0 > 0 ? S.rn / S.rn0 : 0.0;
  return NB_OK;
}

int nb_batch_cycles(const nb_batch *b, int *cycles) {
  clear_status();
  if (!b) return fail(NB_ERR_HANDLE, "null batch");
  int v = 0;
  cudaStream_t s = lib_stream();
  NB_CUDA(cudaMemcpyAsync(&v, b->B.cycles, sizeof(int), cudaMemcpyDeviceToHost, s));
  NB_TRY(device_error_check(s));
  if (cycles) *cycles = v;
  return NB_OK;
}

// Host <-> device copies of the concatenated right-hand side and solution
// (problem p at nb_batch_problem's offset), asynchronous on the library
// stream: host buffers should be pinned.
int nb_batch_rhs_in(nb_batch *b, const double *f_host) {
  clear_status();
  if (!b || !f_host) return fail(NB_ERR_ARG, "nb_batch_rhs_in: null argument");
  NB_CUDA(cudaMemcpyAsync(b->B.f, f_host, b->B.n * sizeof(double), cudaMemcpyHostToDevice,
                          lib_stream()));
  return NB_OK;
}

int nb_batch_x_out(nb_batch *b, double *x_host) {
  clear_status();
  if (!b || !x_host) return fail(NB_ERR_ARG, "nb_batch_x_out: null argument");
  NB_CUDA(cudaMemcpyAsync(x_host, b->B.x, b->B.n * sizeof(double), cudaMemcpyDeviceToHost,
                          lib_stream()));
  return NB_OK;
}

}  // extern "C"

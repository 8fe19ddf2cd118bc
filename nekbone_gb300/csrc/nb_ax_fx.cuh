// nb_ax_fx.cuh -- the FP64 element operator (ax_e, cg.f:142-168, with
// local_grad3 / local_grad3_t, cg.f:170-212) evaluated in 64-bit fixed
// point on the integer pipes instead of GB300's FP64 pipe.
//
// GB300 executes about 0.5e12 FP64 fused multiply-adds per second, but
// about 14e12 32x32->64-bit integer multiply-adds (mad.wide.s32) and 19e12
// simple integer operations (measured).  A product of two 60-bit
// fixed-point numbers built from three integer multiply-adds therefore
// costs a tenth of one DFMA.  So this operator keeps its values as block-floating-point
// integers and leaves only the CG vector arithmetic (p update, +0.1 p, pap)
// on the FP64 pipe:
//
//  * each element's input p is scaled by one power of two chosen from the
//    element's largest exponent and rounded to an integer P, |P| < 2^59
//    (to_fixed); the derivative tables are fixed-point integers with FC
//    fractional bits (|C| <= 2^59, rounded once on the host from D's exact
//    value); the metric g is converted once per solve, one exponent per
//    element (|G| < 2^60);
//  * a product a*b of two such integers is formed from balanced 32-bit
//    halves, a = ah 2^32 + al with al in [-2^31, 2^31):
//        a*b ~= ah*bh 2^64 + (ah*bl + al*bh) 2^32,
//    al*bl (|al*bl| <= 2^62, unbiased: al is symmetric) dropped.  In the
//    metric step the terms of one output are accumulated in int64 registers
//    (Acc) and combined once, rounded to units of 2^64 (hh + x / 2^32: the
//    high word of x, no shift; x starts at half a unit), so one output's
//    error is about one unit, ~2^-55 of its largest product -- the FP64
//    evaluation's own rounding of a 6-term sum.  In the six contraction
//    stages each cross term is a 32-bit mad.hi (its high word, units of
//    2^64) and the floors' mean loss is added back once (AccH): a few
//    units per output, for a fifth fewer instructions;
//  * the even-odd split of the GLL derivative (as k_ax_eo) halves the
//    products: per point and direction 6 multiply-adds at lx1 = 12;
//  * after the gradient and after the metric step the element's values are
//    renormalised by one shift (the element-wide OR of the magnitudes gives
//    the top bit), so every stage starts from ~58 significant bits of the
//    element's largest value;
//  * the result goes back to FP64 rounded to nearest even by the
//    integer-to-FP64 conversion (one FP64-pipe operation a point) and an
//    exact move of the exponent field; the input goes in by an exact FP64
//    scaling and the FP64-to-integer conversion (two more), where the FP64
//    pipe has room beside the integer work.
// This is block floating point: the error of a value is bounded relative to
// the largest value of its element (~2^-56), where FP64 bounds it relative
// to the value itself.  Results agree with the reference's FP64 evaluation
// to rounding (~1e-15 of the element's scale), not bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nb_kernels.cuh"

// CTAs per SM of the fixed-point operator at lx1 <= 12: its three
// shared-memory arrays (42 KB at lx1 = 12) allow five, and the bound keeps
// the registers within five (1.90 ms at 32^3, against 2.01 ms with four
// arrays and four CTAs, 2.25 ms with rows padded to lx1 + 1 and three).
// The output rows of a line are unrolled two at a time (fully unrolled,
// the kernel spills and measures slower).
#ifndef NB_FX_MINB
#define NB_FX_MINB 5
#endif
#ifndef NB_FX_AUNROLL
#define NB_FX_AUNROLL 2
#endif
#define NB_FX_PRAGMA(x) _Pragma(#x)
#define NB_FX_UNROLL(n) NB_FX_PRAGMA(unroll n)

namespace nb {
namespace fx {

typedef long long i64;
typedef unsigned long long u64;

// ------------------------------------------------------------ integers --
// balanced halves: x = hi * 2^32 + lo, lo in [-2^31, 2^31)
struct Sp {
  int lo, hi;
};
__device__ __forceinline__ Sp split(i64 x) {
  Sp s;
  const unsigned low = unsigned(u64(x));
  s.lo = int(low);
  s.hi = int(u64(x) >> 32) + int(low >> 31);
  return s;
}

// A sum of products a*b in units of 2^64: hh counts ah*bh, x and x2 count
// ah*bl and al*bh in units of 2^32 (two accumulators: two dependency chains
// of half the length), x started at half a unit so that the high word of
// x + x2 rounds to nearest (al*bl dropped).  Each product is one 32x32 ->
// 64-bit multiply-add (mad.wide.s32), written in C++ so that a coefficient
// can stay a constant-bank operand.
struct Acc {
  i64 hh, x, x2;
  __device__ __forceinline__ Acc() : hh(0), x(1ll << 31), x2(0) {}
  __device__ __forceinline__ void mac(int chi, int clo, const Sp &v) {
    hh += i64(chi) * i64(v.hi);
    x += i64(chi) * i64(v.lo);
    x2 += i64(clo) * i64(v.hi);
  }
  __device__ __forceinline__ void mac(const Sp &c, const Sp &v) { mac(c.hi, c.lo, v); }
  __device__ __forceinline__ i64 result() const { return hh + ((x + x2) >> 32); }
};

// The same sum with the two cross terms taken as high words only: each
// ah*bl and al*bh is one 32-bit mad.hi (floor of the product / 2^32, in
// units of 2^64) instead of a 64-bit mad.wide, and the floors' average loss
// of half a unit each is added back once (not for an all-zero sum, so that
// A 0 = 0 stays exact).  An output's error grows from about one unit to a
// few; in the contraction stages, where this form is used, the operator's
// difference from the FP64 reference evaluation stays within 10 % of the
// exact-cross-term form's (3.1e-15 instead of 2.8e-15 of max|w| at lx1 = 12,
// deformed), and the operator takes 1.63 instead of 1.88 ms at 32^3.  The
// metric step keeps Acc: its cross terms carry the error into every later
// stage (8e-15 with mad.hi there).
struct AccH {
  i64 hh;
  int x, x2;  // high words below 2^27 (|ah| < 2^28, |al| <= 2^31); the
              // lx1/2 <= 8 of them and x + x2 stay below 2^31
  __device__ __forceinline__ AccH() : hh(0), x(0), x2(0) {}
  __device__ __forceinline__ void mac(int chi, int clo, const Sp &v) {
    hh += i64(chi) * i64(v.hi);
    x = __mulhi(chi, v.lo) + x;
    x2 = __mulhi(clo, v.hi) + x2;
  }
  // nmac multiply-adds were made
  __device__ __forceinline__ i64 result(int nmac) const {
    return hh + i64(x + x2 + ((x | x2) != 0 ? nmac : 0));
  }
};

// v * 2^sh for 0 <= sh < 64: the operator's two renormalisation shifts are
// never negative.  After the gradient every output is below 2^58.6 (six
// products of |C| <= 2^59 and an even-odd sum below 2^60, in units of 2^64,
// twice), so its shift is >= 0; after the metric step every output is below
// 2^56.6 (three products of |G| < 2^60 and a value below 2^59), so its shift
// is >= 2.  The operator checks both and reports a violation through the
// device error word.
__device__ __forceinline__ i64 shift_up(i64 v, int sh) { return i64(u64(v) << sh); }

// ----------------------------------------------------- FP64 <-> fixed --
__device__ __forceinline__ int bexp(double x) {
  return int((u64(__double_as_longlong(x)) >> 52) & 0x7FFu);
}

// x * 2^(1075 - emax + up) rounded to nearest (ties away from zero), for x
// whose biased exponent is <= emax: |result| < 2^(53 + up).  This and
// to_double are the conversions' fallbacks for exponents out of the fast
// forms' range; out of line, they leave the operator's code smaller (100 CG
// iterations at 32^3: 247.0 instead of 248.3 ms).
static __device__ __noinline__ i64 to_fixed(double x, int emax, int up) {
  const u64 b = u64(__double_as_longlong(x));
  const int e = int((b >> 52) & 0x7FFu);
  const u64 m = (b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  const int sh = (e ? e : 1) - emax + up;
  u64 mag;
  if (sh >= 0) mag = m << sh;
  else if (sh > -54) mag = ((m >> (-sh - 1)) + 1ull) >> 1;
  else mag = 0ull;
  return (b >> 63) ? -i64(mag) : i64(mag);
}

// W * 2^s rounded to the nearest FP64 value (ties to even)
static __device__ __noinline__ double to_double(i64 W, int s) {
  if (W == 0) return 0.0;
  const u64 sign = u64(W) & (1ull << 63);
  u64 mag = W < 0 ? u64(-W) : u64(W);
  const int lz = __clzll(i64(mag));
  mag <<= lz;                       // top bit at 63
  int ex = 63 - lz + s;             // unbiased exponent of the value
  u64 mant = mag >> 11;             // 53 bits
  const u64 rem = mag & 0x7FFull;
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ++mant;
  if (mant >> 53) {
    mant >>= 1;
    ++ex;
  }
  int be = ex + 1023;
  if (be >= 2047) return __longlong_as_double(i64(sign | (0x7FFull << 52)));
  if (be <= 0) {  // subnormal: mant * 2^(ex - 52) with 2^-1074 as the unit
    const int rs = 1 - be;
    if (rs > 53) return __longlong_as_double(i64(sign));
    const u64 half = 1ull << (rs - 1), low = mant & ((1ull << rs) - 1ull);
    u64 q = mant >> rs;
    if (low > half || (low == half && (q & 1ull))) ++q;
    return __longlong_as_double(i64(sign | q));
  }
  return __longlong_as_double(i64(sign | (u64(be) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}


// W * 2^s, bitwise as to_double: the integer-to-FP64 conversion rounds |W|
// to 53 bits to nearest even, as to_double does, and the exponent field is
// then moved by s exactly; results that would be subnormal or overflow take
// to_double.  One FP64-pipe conversion instead of ~25 integer instructions
// (1.93 -> 1.88 ms for the operator at 32^3; the same conversion for
// to_fixed, at two FP64-pipe operations a value, changes the rounding of
// ties and was not kept).
__device__ __forceinline__ double to_double_cvt(i64 W, int s) {
  const double d = __ll2double_rn(W);
  const i64 b = __double_as_longlong(d);
  const int e = int((b >> 52) & 0x7FF);
  const int e2 = e + s;
  if (d != 0.0 && e2 >= 1 && e2 <= 2046) return __longlong_as_double(b + (i64(s) << 52));
  return d == 0.0 ? 0.0 : to_double(W, s);
}
// x * 2^(1075 - emax + up) rounded to the nearest integer, ties to even
// (to_fixed rounds them away from zero), by an exact FP64 scaling and the
// FP64-to-integer conversion: two FP64-pipe operations instead of ~15
// integer instructions (1.63 -> 1.61 ms for the operator at 32^3)
__device__ __forceinline__ i64 to_fixed_cvt(double x, int emax, int up) {
  const int k = 1075 - emax + up;
  if (k > 1023 || k < -1022) return to_fixed(x, emax, up);  // 2^k not a normal double
  const double sc = __longlong_as_double(i64(k + 1023) << 52);
  return __double2ll_rn(x * sc);
}
// ----------------------------------------------------- block reductions --
// lanes of warp w of an nt-thread block
__device__ __forceinline__ unsigned warp_mask(int nt, int w) {
  const int n = nt - 32 * w;
  return n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
}

// ------------------------------------------------------------ operator --
// Derivative tables in fixed point: E, O of D, then E, O of D^T (the
// even-odd tables of k_ax_eo, 4*(lx1/2)^2 values, row a), as balanced
// halves, |coefficient| <= 2^59.  A kernel parameter, read as multiply-add
// operands.
template <int LX>
struct FxCoef {
  int hi[4 * (LX / 2) * (LX / 2)];
  int lo[4 * (LX / 2) * (LX / 2)];
  int fc;  // fractional bits: coefficient = (hi 2^32 + lo) 2^-fc
};

template <int LX>
struct FxShared {
  static constexpr int N = (LX * LX + 1) * LX;
  i64 A[N];
  i64 C[N];
  i64 D[N];
  int emax[8];
  unsigned orl[8], orh[8];
  double red[32];
};

// Element arrays in shared memory: rows of lx1 8-byte words, planes lx1^2 + 1
// words apart.  The plane pitch is 1 modulo 16, so the r-lines that 16
// consecutive threads start (thread t: j = t / lx1, k = t mod lx1) fall on
// distinct banks; so do the own columns (i + lx1 j).
template <int LX>
__device__ __forceinline__ int fx_at(int i, int j, int k) {
  return i + LX * j + (LX * LX + 1) * k;
}

// y(0..n-1) = C v of one line v (fixed point, |v| < 2^59), coefficient
// tables at offset q0 of cf (E at q0, O at q0 + h^2); y in units of 2^64 of
// the products (|y| < 2^58.6), handed to put(m, y(m)) as soon as each pair
// y(a), y(n-1-a) is formed (no output array stays live)
template <int LX, typename Put>
__device__ __forceinline__ void fx_line(const i64 *v, const FxCoef<LX> &cf, int q0, Put put) {
  constexpr int H = LX / 2;
  Sp ve[H], vo[H];
#pragma unroll
  for (int m = 0; m < H; ++m) {
    ve[m] = split(v[m] + v[LX - 1 - m]);
    vo[m] = split(v[m] - v[LX - 1 - m]);
  }
  NB_FX_UNROLL(NB_FX_AUNROLL)
  for (int a = 0; a < H; ++a) {
    AccH e, o;
#pragma unroll
    for (int m = 0; m < H; ++m) {
      const int qe = q0 + a * H + m, qo = qe + H * H;
      e.mac(cf.hi[qe], cf.lo[qe], ve[m]);
      o.mac(cf.hi[qo], cf.lo[qo], vo[m]);
    }
    const i64 ye = e.result(H), yo = o.result(H);
    put(a, ye + yo);
    put(LX - 1 - a, yo - ye);
  }
}

// OR of the magnitudes of a thread's values, combined over the block after
// the next __syncthreads (fx_or_read): its top bit is the largest's
__device__ __forceinline__ void fx_or_post(u64 v, unsigned *orl, unsigned *orh, int t, int nt) {
  const int w = t >> 5;
  const unsigned msk = warp_mask(nt, w);
  const unsigned l = __reduce_or_sync(msk, unsigned(v)), h = __reduce_or_sync(msk, unsigned(v >> 32));
  if ((t & 31) == 0) {
    orl[w] = l;
    orh[w] = h;
  }
}
// the shift that brings the block's largest magnitude below 2^59
__device__ __forceinline__ int fx_or_shift(const unsigned *orl, const unsigned *orh, int nt) {
  u64 v = 0;
  for (int w = 0; w < (nt + 31) / 32; ++w) v |= (u64(orh[w]) << 32) | orl[w];
  if (v == 0) return 0;
  return 58 - (63 - __clzll(i64(v)));
}
// one's complement magnitude: the same top bit as |v| (one lower for an
// exact negative power of two, which the bounds leave room for)
__device__ __forceinline__ u64 mag(i64 v) { return u64(v ^ (v >> 63)); }

// MODE 0 / 1 / 2 as k_ax_eo (AxArgs); a.gfx / a.gexp hold the metric in
// fixed point (metric_fx_prepare).
template <int LX, int MODE>
__device__ __forceinline__ void ax_fx_body(const AxArgs<double> &a, const FxCoef<LX> &cf) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  FxShared<LX> &sm = *reinterpret_cast<FxShared<LX> *>(smem_raw);
  constexpr int L2 = LX * LX, L3 = LX * LX * LX, H = LX / 2;
  const int t = threadIdx.x + LX * threadIdx.y;
  const int i = threadIdx.x, j = threadIdx.y;  // own column (i,j)
  const int e = blockIdx.x;
  const size_t base = size_t(e) * L3;
  const int fc = cf.fc;
  if (a.act && !a.act[size_t(a.el_prob[e]) * a.act_stride]) return;  // the whole CTA

  // direction update (MODE 1) / correction (MODE 2), in FP64, then the
  // element's exponent and its fixed-point block
  int em = 0;
  {
    double uk[LX];
    double pold[LX];
    const double beta = (MODE == 1 && !a.first) ? a.sc->beta : 0.0;
#pragma unroll
    for (int k = 0; k < LX; ++k) {  // all loads before the first store
      const size_t id = base + size_t(k) * L2 + t;
      if (MODE == 1) {
        uk[k] = a.u[id];
        pold[k] = a.first ? 0.0 : a.pold[id];
      } else if (MODE == 2) {
        uk[k] = a.p[id];
        pold[k] = a.e ? double(a.e[id]) : 0.0;
      } else {
        uk[k] = a.u[id];
      }
    }
#pragma unroll
    for (int k = 0; k < LX; ++k) {
      const size_t id = base + size_t(k) * L2 + t;
      if (MODE == 1) {
        if (!a.first) uk[k] = fma_rn(beta, pold[k], uk[k]);  // add2s1, math.f:534
        a.p[id] = uk[k];
      } else if (MODE == 2 && a.e) {
        uk[k] = fma_rn(a.scale, pold[k], uk[k]);
        a.p[id] = uk[k];
      }
    }
#pragma unroll
    for (int k = 0; k < LX; ++k) em = max(em, bexp(uk[k]));
    const int w = t >> 5;
    const int r = __reduce_max_sync(warp_mask(L2, w), unsigned(em));
    if ((t & 31) == 0) sm.emax[w] = r;
    __syncthreads();
    em = 0;
    for (int q = 0; q < (L2 + 31) / 32; ++q) em = max(em, sm.emax[q]);
#pragma unroll
    for (int k = 0; k < LX; ++k) sm.A[fx_at<LX>(i, j, k)] = to_fixed_cvt(uk[k], em, 6);
  }
  const int sP = em - 1081;  // p = P 2^sP
  __syncthreads();

  // Thread (i,j) takes, in each contraction stage, the r-line (j, k=i),
  // the s-line (i, k=j) and its own column, the t-line (i,j): one loop over
  // the three directions with run-time strides keeps one copy of the line
  // code per stage; every output goes to shared memory.
  const int lb0 = fx_at<LX>(0, j, i), lb1 = fx_at<LX>(i, 0, j), lb2 = fx_at<LX>(i, j, 0);

  // gradient (local_grad3): A -> C (us), D (ut); then, once every s- and
  // t-line of A was read, A -> A (ur) line by line in place
  u64 orv = 0;
#pragma unroll 1
  for (int dd = 0; dd < 3; ++dd) {
    const int d = dd == 2 ? 0 : dd + 1;
    if (dd == 2) __syncthreads();
    const int b0 = d == 0 ? lb0 : d == 1 ? lb1 : lb2;
    const int st = d == 0 ? 1 : d == 1 ? LX : (LX * LX + 1);
    i64 *out = d == 0 ? sm.A : d == 1 ? sm.C : sm.D;
    i64 v[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = sm.A[b0 + m * st];
    fx_line<LX>(v, cf, 0, [&](int m, i64 y) {
      out[b0 + m * st] = y;
      orv |= mag(y);
    });
  }
  fx_or_post(orv, sm.orl, sm.orh, t, L2);
  __syncthreads();
  int s1 = fx_or_shift(sm.orl, sm.orh, L2);
  if (s1 < 0) {  // outside the bounds shift_up relies on: results invalid
    if (t == 0 && a.err) atomicOr(a.err, 2u);
    s1 = 0;
  }
  const int sU = sP - fc + 64 - s1;  // ur = UR 2^sU after the shift

  // metric (cg.f:156-163) at the thread's own points, in place
  const int eg = a.gexp[e];
  const int sW = 64 + (eg - 1082) + sU;  // wr = WR 2^sW before renormalising
  orv = 0;
#pragma unroll 4
  for (int k = 0; k < LX; ++k) {
    const int q = fx_at<LX>(i, j, k);
    const Sp ur = split(shift_up(sm.A[q], s1)), us = split(shift_up(sm.C[q], s1)),
             ut = split(shift_up(sm.D[q], s1));
    const int4 *gp = reinterpret_cast<const int4 *>(a.gfx + 6 * (base + size_t(k) * L2 + t));
    const int4 g01 = __ldg(gp), g23 = __ldg(gp + 1), g45 = __ldg(gp + 2);
    const Sp G1 = {g01.x, g01.y}, G2 = {g01.z, g01.w}, G3 = {g23.x, g23.y},
             G4 = {g23.z, g23.w}, G5 = {g45.x, g45.y}, G6 = {g45.z, g45.w};
    Acc wr, ws, wt;
    wr.mac(G1, ur); wr.mac(G2, us); wr.mac(G3, ut);
    ws.mac(G2, ur); ws.mac(G4, us); ws.mac(G5, ut);
    wt.mac(G3, ur); wt.mac(G5, us); wt.mac(G6, ut);
    const i64 r_ = wr.result(), s_ = ws.result(), t_ = wt.result();
    sm.A[q] = r_;
    sm.C[q] = s_;
    sm.D[q] = t_;
    orv |= mag(r_) | mag(s_) | mag(t_);
  }
  fx_or_post(orv, sm.orl, sm.orh, t, L2);
  __syncthreads();
  int s2 = fx_or_shift(sm.orl, sm.orh, L2);
  if (s2 < 0) {  // as s1
    if (t == 0 && a.err) atomicOr(a.err, 2u);
    s2 = 0;
  }
  const int sT = 64 - fc + sW - s2;  // transposed-gradient outputs: value 2^sT

  // transposed gradient (local_grad3_t) with D^T, each line in place: A
  // (tr), C (ts), D (tt); a thread reads and writes only its own lines
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    const int b0 = d == 0 ? lb0 : d == 1 ? lb1 : lb2;
    const int st = d == 0 ? 1 : d == 1 ? LX : (LX * LX + 1);
    i64 *out = d == 0 ? sm.A : d == 1 ? sm.C : sm.D;
    const i64 *src = out;
    i64 v[LX];
#pragma unroll
    for (int m = 0; m < LX; ++m) v[m] = shift_up(src[b0 + m * st], s2);
    fx_line<LX>(v, cf, 2 * H * H, [&](int m, i64 y) { out[b0 + m * st] = y; });
  }
  __syncthreads();

  // w_L = tr + ts + tt in FP64; the CG epilogue as k_ax_eo's.  The
  // interior's p (written above by this thread, so in cache), c and f are
  // read again here rather than held in registers through the contractions.
  const bool col_interior = (i > 0) && (i < LX - 1) && (j > 0) && (j < LX - 1);
  double part = 0.0;
  double pk[LX], ck[LX], fk[LX];
  if (MODE != 0 && col_interior) {
#pragma unroll
    for (int k = 1; k < LX - 1; ++k) {  // all loads before the first store
      const size_t id = base + size_t(k) * L2 + t;
      pk[k] = a.p[id];
      ck[k] = __ldg(a.c + id);
      if (MODE == 2) fk[k] = __ldg(a.f + id);
    }
  }
#pragma unroll
  for (int k = 0; k < LX; ++k) {
    const int q = fx_at<LX>(i, j, k);
    double wl = to_double_cvt(sm.A[q] + sm.C[q] + sm.D[q], sT);
    const size_t id = base + size_t(k) * L2 + t;
    const bool interior = col_interior && (k > 0) && (k < LX - 1);
    if (MODE == 1) {
      if (interior) {
        wl = fma_rn(0.1, pk[k], wl);
        part = fma_rn(mul_rn(wl, ck[k]), pk[k], part);
      }
      a.w[id] = wl;
    } else if (MODE == 2) {
      if (interior) {
        const double rv = fk[k] - fma_rn(0.1, pk[k], wl);
        a.r[id] = rv;
        part = fma_rn(mul_rn(rv, ck[k]), rv, part);
      } else {
        a.w[id] = wl;
      }
    } else {
      a.w[id] = wl;
    }
  }
  if (MODE != 0) {
    const double s = block_sum<double>(part, sm.red);
    if (t == 0) a.partial[e] = s;
  }
}

// (the thread bound is the whole warps the block occupies, so that the
// register budget per thread is what NB_FX_MINB resident blocks leave)
template <int LX, int MODE>
__global__ void __launch_bounds__((LX * LX + 31) / 32 * 32, (LX <= 12 ? NB_FX_MINB : 1))
    k_ax_fx(AxArgs<double> a, const __grid_constant__ FxCoef<LX> cf) {
  ax_fx_body<LX, MODE>(a, cf);
}

template <int LX>
constexpr size_t ax_fx_smem_bytes() {
  return sizeof(FxShared<LX>);
}

}  // namespace fx
}  // namespace nb

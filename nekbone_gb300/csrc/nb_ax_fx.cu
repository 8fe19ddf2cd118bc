// nb_ax_fx.cu -- set-up of the fixed-point FP64 element operator
// (nb_ax_fx.cuh): its derivative tables, computed exactly on the host, and
// the per-solve conversion of the metric g into fixed point.
#include <cmath>
#include <cstdint>
#include <vector>

#include "nb_ax_fx.cuh"
#include "nb_solver.h"

namespace nb {

namespace {

typedef __int128 i128;

// x = m 2^e exactly, |m| < 2^53
void decompose(double x, int64_t *m, int *e) {
  if (x == 0.0) {
    *m = 0;
    *e = 0;
    return;
  }
  int ex = 0;
  const double fr = std::frexp(x, &ex);
  *m = int64_t(std::ldexp(fr, 53));
  *e = ex - 53;
}

// round((a + sgn b) 2^sh) to the nearest integer (ties to even), from the
// exact values of a and b (a term below 2^-70 of the other is dropped)
int64_t scaled_sum(double a, double b, int sgn, int sh) {
  int64_t ma, mb;
  int ea, eb;
  decompose(a, &ma, &ea);
  decompose(b, &mb, &eb);
  if (ma == 0) ea = eb;
  if (mb == 0) eb = ea;
  if (ea - eb > 70) mb = 0, eb = ea;
  if (eb - ea > 70) ma = 0, ea = eb;
  const int e0 = ea < eb ? ea : eb;
  const i128 T = (i128(ma) << (ea - e0)) + i128(sgn) * (i128(mb) << (eb - e0));
  const int s = e0 + sh;
  if (s >= 0) return int64_t(T << s);
  if (-s > 120) return 0;
  const i128 neg = T < 0 ? -T : T;
  i128 q = neg >> (-s);
  const i128 rem = neg - (q << (-s)), half = i128(1) << (-s - 1);
  if (rem > half || (rem == half && (q & 1))) ++q;
  return int64_t(T < 0 ? -q : q);
}

// one block per element: the element's largest exponent over its 6 lx1^3
// metric values, then each value as balanced halves of g 2^(1082 - emax)
__global__ void __launch_bounds__(256)
    k_metric_fx(const double *__restrict__ g, int2 *__restrict__ gfx, int *__restrict__ gexp,
                int blk) {
  __shared__ int wmax[8];
  const int t = threadIdx.x;
  const size_t base = size_t(blockIdx.x) * blk;
  int em = 0;
  for (int q = t; q < blk; q += 256) em = max(em, fx::bexp(g[base + q]));
  const int r = __reduce_max_sync(0xFFFFFFFFu, unsigned(em));
  if ((t & 31) == 0) wmax[t >> 5] = r;
  __syncthreads();
  em = 0;
  for (int w = 0; w < 8; ++w) em = max(em, wmax[w]);
  for (int q = t; q < blk; q += 256) {
    const fx::Sp s = fx::split(fx::to_fixed(g[base + q], em, 7));
    gfx[base + q] = make_int2(s.lo, s.hi);
  }
  if (t == 0) gexp[blockIdx.x] = em;
}

}  // namespace

// E, O of D and of D^T (even_odd_tables' order and meaning) in fixed point
// with fc fractional bits, |C| <= 2^59, split into balanced halves.
bool fx_tables(const std::vector<double> &D, int lx, std::vector<int> &hi,
               std::vector<int> &lo, int *fc) {
  if (lx % 2 != 0 || lx < 2) return false;
  const int h = lx / 2;
  auto Dm = [&](int r, int c) { return D[r + c * lx]; };
  double mx = 0.0;
  for (int a = 0; a < h; ++a)
    for (int m = 0; m < h; ++m) {
      mx = std::max(mx, std::fabs(Dm(a, m) + Dm(a, lx - 1 - m)) / 2);
      mx = std::max(mx, std::fabs(Dm(a, m) - Dm(a, lx - 1 - m)) / 2);
      mx = std::max(mx, std::fabs(Dm(m, a) + Dm(lx - 1 - m, a)) / 2);
      mx = std::max(mx, std::fabs(Dm(m, a) - Dm(lx - 1 - m, a)) / 2);
    }
  if (!(mx > 0.0)) return false;
  int k = 0;
  std::frexp(mx * (1.0 + 1e-15), &k);  // mx < 2^k
  *fc = 59 - k;
  hi.assign(4 * h * h, 0);
  lo.assign(4 * h * h, 0);
  auto put = [&](int q, double x1, double x2, int sgn) {
    const int64_t C = scaled_sum(x1, x2, sgn, *fc - 1);
    const int32_t l = int32_t(uint32_t(uint64_t(C)));
    lo[q] = l;
    hi[q] = int32_t((C - int64_t(l)) >> 32);
  };
  for (int a = 0; a < h; ++a)
    for (int m = 0; m < h; ++m) {
      put(a * h + m, Dm(a, m), Dm(a, lx - 1 - m), 1);
      put(h * h + a * h + m, Dm(a, m), Dm(a, lx - 1 - m), -1);
      put(2 * h * h + a * h + m, Dm(m, a), Dm(lx - 1 - m, a), 1);
      put(3 * h * h + a * h + m, Dm(m, a), Dm(lx - 1 - m, a), -1);
    }
  return true;
}

void metric_fx_invalidate(const Operator &op) { op.gfx_src = nullptr; }

int metric_fx_prepare(const Operator &op, const double *g, cudaStream_t s) {
  if (op.gfx_src == g && op.gfx) return NB_OK;
  const long nv = 6 * op.n;
  if (op.gfx_cap < nv) {
    if (op.gfx) cudaFree(op.gfx);
    if (op.gexp) cudaFree(op.gexp);
    op.gfx = nullptr;
    op.gexp = nullptr;
    op.gfx_cap = 0;
    NB_CUDA(cudaMalloc(&op.gfx, size_t(nv) * sizeof(int2)));
    NB_CUDA(cudaMalloc(&op.gexp, size_t(op.nelt) * sizeof(int)));
    op.gfx_cap = nv;
  }
  const int blk = 6 * op.lx * op.lx * op.lx;
  k_metric_fx<<<op.nelt, 256, 0, s>>>(g, op.gfx, op.gexp, blk);
  NB_CUDA(cudaGetLastError());
  op.gfx_src = g;
  return NB_OK;
}

}  // namespace nb

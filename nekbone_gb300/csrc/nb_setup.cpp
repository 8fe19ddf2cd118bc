// nb_setup.cpp -- host-side set-up math of the nekbone_gb300 library.
//
// Gauss-Lobatto-Legendre points and weights (speclib.f ZWGLL -> ZWGLJD ->
// ZWGJD -> JACG -> JACOBF, ENDW1/ENDW2, GAMMAF, PNORMJ), the 1-D spectral
// matrices (semhat.f), the box global numbering (prox_dssum.f set_vert_box),
// the element decomposition (driver.f cubic), the jl local gather-scatter
// topology (jl/gs.c nonzero_ids + local_map) and the generalized symmetric
// eigensolver that hsmg's fast-diagonalisation set-up needs (hsmg.f:483-523).
// These run once per mesh; the per-iteration work is in the CUDA sources.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nb_internal.h"

namespace nb {

namespace {

// GAMMAF, speclib.f:371-393: exact values at the half-integers and small
// integers that the GLL/GJ formulas need.
double gamma_tab(double x) {
  const double pi = 4.0 * std::atan(1.0);
  double g = 1.0;
  if (x == -0.5) g = -2.0 * std::sqrt(pi);
  if (x == 0.5) g = std::sqrt(pi);
  if (x == 1.0) g = 1.0;
  if (x == 2.0) g = 1.0;
  if (x == 1.5) g = std::sqrt(pi) / 2.;
  if (x == 2.5) g = 1.5 * std::sqrt(pi) / 2.;
  if (x == 3.5) g = 0.5 * (2.5 * (1.5 * std::sqrt(pi)));
  if (x == 3.) g = 2.;
  if (x == 4.) g = 6.;
  if (x == 5.) g = 24.;
  if (x == 6.) g = 120.;
  return g;
}

// Jacobi polynomial P_n^{(a,b)}(x), its derivative, and the previous degree's
// values (JACOBF, speclib.f:479-518; three-term recurrence).
struct Jacobi {
  double p, pd, pm1, pdm1;
};
Jacobi jacobi(int n, double a, double b, double x) {
  Jacobi r{1.0, 0.0, 0.0, 0.0};
  if (n == 0) return r;
  const double apb = a + b;
  double pl = r.p, pdl = r.pd;
  r.p = (a - b + (apb + 2.) * x) / 2.;
  r.pd = (apb + 2.) / 2.;
  if (n == 1) return r;
  for (int k = 2; k <= n; ++k) {
    const double dk = k;
    const double a1 = 2. * dk * (dk + apb) * (2. * dk + apb - 2.);
    const double a2 = (2. * dk + apb - 1.) * (a * a - b * b);
    const double b3 = (2. * dk + apb - 2.);
    const double a3 = b3 * (b3 + 1.) * (b3 + 2.);
    const double a4 = 2. * (dk + a - 1.) * (dk + b - 1.) * (2. * dk + apb);
    const double pn = ((a2 + a3 * x) * r.p - a4 * pl) / a1;
    const double pdn = ((a2 + a3 * x) * r.pd - a4 * pdl + a3 * r.p) / a1;
    pl = r.p;
    r.p = pn;
    pdl = r.pd;
    r.pd = pdn;
  }
  r.pm1 = pl;
  r.pdm1 = pdl;
  return r;
}

// Zeros of P_np^{(a,b)} by Newton with deflation from Chebyshev-Gauss
// guesses (JACG, speclib.f:421-477: EPS=1e-12, at most 10 steps), sorted.
void jacobi_zeros(double *x, int np, double a, double b) {
  const int n = np - 1;
  const double dth = 4. * std::atan(1.0) / (2. * double(n) + 2.);
  double xlast = 0.0;
  for (int j = 1; j <= np; ++j) {
    const double xc = std::cos((2. * (double(j) - 1.) + 1.) * dth);
    double xx = j == 1 ? xc : (xc + xlast) / 2.;
    for (int k = 0; k < 10; ++k) {
      const Jacobi jp = jacobi(np, a, b, xx);
      double rs = 0.;
      for (int i = 1; i <= j - 1; ++i) rs = rs + 1. / (xx - x[np - i]);
      const double dx = -jp.p / (jp.pd - rs * jp.p);
      xx = xx + dx;
      if (std::fabs(dx) < 1.0e-12) break;
    }
    x[np - j] = xx;
    xlast = xx;
  }
  // selection sort, ascending (speclib.f:463-476)
  for (int i = 0; i < np; ++i) {
    double xmin = 2.;
    int jmin = i;
    for (int j = i; j < np; ++j)
      if (x[j] < xmin) {
        xmin = x[j];
        jmin = j;
      }
    if (jmin != i) std::swap(x[i], x[jmin]);
  }
}

double pnormj(int n, double a, double b) {
  const double dn = n, c = a + b + 1.;
  double prod;
  if (n <= 1) {
    prod = gamma_tab(dn + a) * gamma_tab(dn + b);
    prod = prod / (gamma_tab(dn) * gamma_tab(dn + a + b));
    return prod * std::pow(2., c) / (2. * dn + c);
  }
  prod = gamma_tab(a + 1.) * gamma_tab(b + 1.);
  prod = prod / (2. * (1. + c) * gamma_tab(c + 1.));
  prod = prod * (1. + a) * (2. + a);
  prod = prod * (1. + b) * (2. + b);
  for (int i = 3; i <= n; ++i) {
    const double di = i;
    prod = prod * ((di + a) * (di + b) / (di * (di + a + b)));
  }
  return prod * std::pow(2., c) / (2. * dn + c);
}

// Gauss-Jacobi points and weights (ZWGJD, speclib.f:155-205)
void gauss_jacobi(double *z, double *w, int np, double a, double b) {
  const double apb = a + b;
  if (np == 1) {
    z[0] = (b - a) / (apb + 2.);
    w[0] = gamma_tab(a + 1.) * gamma_tab(b + 1.) / gamma_tab(apb + 2.) *
           std::pow(2., apb + 1.);
    return;
  }
  jacobi_zeros(z, np, a, b);
  const int n = np - 1;
  const double dnp1 = n + 1, dnp2 = n + 2;
  const double fac1 = dnp1 + a + b + 1.;
  const double fac2 = fac1 + dnp1;
  const double fac3 = fac2 + 1.;
  const double fnorm = pnormj(n + 1, a, b);
  const double rcoef = (fnorm * fac2 * fac3) / (2. * fac1 * dnp2);
  for (int i = 0; i < np; ++i) {
    const Jacobi jp = jacobi(n + 2, a, b, z[i]);
    w[i] = -rcoef / (jp.p * jp.pdm1);
  }
}

// End-point weights (ENDW1 / ENDW2, speclib.f:283-369).  left selects ENDW1.
double end_weight(int n, double a, double b, bool left) {
  const double apb = a + b;
  if (n == 0) return 0.;
  const double ga = left ? a + 2. : a + 1., gb = left ? b + 1. : b + 2.;
  double f1 = gamma_tab(ga) * gamma_tab(gb) / gamma_tab(apb + 3.);
  f1 = f1 * (apb + 2.) * std::pow(2., apb + 2.) / 2.;
  if (n == 1) return f1;
  double fint1 = gamma_tab(ga) * gamma_tab(gb) / gamma_tab(apb + 3.);
  fint1 = fint1 * std::pow(2., apb + 2.);
  double fint2 = gamma_tab(a + 2.) * gamma_tab(b + 2.) / gamma_tab(apb + 4.);
  fint2 = fint2 * std::pow(2., apb + 3.);
  double f2 = left ? (-2. * (b + 2.) * fint1 + (apb + 4.) * fint2) *
                         (apb + 3.) / 4.
                   : (2. * (a + 2.) * fint1 - (apb + 4.) * fint2) *
                         (apb + 3.) / 4.;
  if (n == 2) return f2;
  double f3 = 0.;
  for (int i = 3; i <= n; ++i) {
    const double di = i - 1;
    const double abn = a + b + di, abnn = abn + di;
    const double a1 = -(2. * (di + a) * (di + b)) / (abn * abnn * (abnn + 1.));
    const double a2 = (2. * (a - b)) / (abnn * (abnn + 2.));
    const double a3 = (2. * (abn + 1.)) / ((abnn + 2.) * (abnn + 1.));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

}  // namespace

// ZWGLL (speclib.f:107-122) through ZWGLJD (speclib.f:238-281).
void zwgll(double *z, double *w, int np) {
  const int n = np - 1;
  if (np < 2) return;
  if (n - 1 > 0) gauss_jacobi(z + 1, w + 1, n - 1, 1., 1.);
  z[0] = -1.;
  z[np - 1] = 1.;
  for (int i = 1; i < np - 1; ++i) w[i] = w[i] / (1. - z[i] * z[i]);
  w[0] = end_weight(n, 0., 0., true) / (2. * jacobi(n, 0., 0., z[0]).pd);
  w[np - 1] =
      end_weight(n, 0., 0., false) / (2. * jacobi(n, 0., 0., z[np - 1]).pd);
}

// Fornberg finite-difference weights on all points (semhat.f:39-93).
// c is (0:n, 0:m), column-major.
void fd_weights_full(double xx, const double *x, int n, int m, double *c) {
  auto C = [&](int j, int k) -> double & { return c[j + k * (n + 1)]; };
  double c1 = 1., c4 = x[0] - xx;
  for (int k = 0; k <= m; ++k)
    for (int j = 0; j <= n; ++j) C(j, k) = 0.;
  C(0, 0) = 1.;
  for (int i = 1; i <= n; ++i) {
    const int mn = std::min(i, m);
    double c2 = 1.;
    const double c5 = c4;
    c4 = x[i] - xx;
    for (int j = 0; j < i; ++j) {
      const double c3 = x[i] - x[j];
      c2 = c2 * c3;
      for (int k = mn; k >= 1; --k)
        C(i, k) = c1 * (k * C(i - 1, k - 1) - c5 * C(i - 1, k)) / c2;
      C(i, 0) = -c1 * c5 * C(i - 1, 0) / c2;
      for (int k = mn; k >= 1; --k) C(j, k) = (c4 * C(j, k) - k * C(j, k - 1)) / c3;
      C(j, 0) = c4 * C(j, 0) / c3;
    }
    c1 = c2;
  }
}

// semhat.f:2-37: a = stiffness, b = GLL weights, c = b*d, d = derivative,
// z = GLL points, all (0:n) or (0:n,0:n) column-major.
void semhat(double *a, double *b, double *c, double *d, double *z, int n) {
  const int np = n + 1;
  std::vector<double> w(2 * np);
  zwgll(z, b, np);
  for (int i = 0; i <= n; ++i) {
    fd_weights_full(z[i], z, n, 1, w.data());
    for (int j = 0; j <= n; ++j) d[i + j * np] = w[j + np];
  }
  for (int j = 0; j <= n; ++j)
    for (int i = 0; i <= n; ++i) {
      double s = 0.;
      for (int k = 0; k <= n; ++k) s = s + d[k + i * np] * b[k] * d[k + j * np];
      a[i + j * np] = s;
      c[i + j * np] = b[i] * d[i + j * np];
    }
}

// mod1, math.f:418-433
int mod1(int i, int n) {
  if (i == 0 || n == 0) return 0;
  return (i + n - 1) % n + 1;
}

// cubic, driver.f:196-247: the most cube-like factorisation np = mx*my*mz
void cubic(int *mx, int *my, int *mz, int np) {
  *mx = np;
  *my = 1;
  *mz = 1;
  double ratio = np;
  const int iroot3 = int(std::pow(double(np), 1. / 3.) + 0.000001);
  for (int iz = iroot3; iz >= 1; --iz) {
    const int myx = np / iz;
    if (np - myx * iz != 0) continue;
    int ix = 0, iy = 0, z = iz;
    const int iroot2 = int(std::pow(double(myx), 1. / 2.) + 0.000001);
    for (int j = iroot2; j >= 1; --j) {
      iy = j;
      ix = myx / iy;
      if (myx - ix * iy == 0) break;
    }
    if (ix < iy) std::swap(ix, iy);
    if (ix < z) std::swap(ix, z);
    if (iy < z) std::swap(iy, z);
    if (double(ix) / z < ratio) {
      ratio = double(ix) / z;
      *mx = ix;
      *my = iy;
      *mz = z;
    }
  }
}

// get_exyz, prox_dssum.f:75-86
void get_exyz(int *ex, int *ey, int *ez, int eg, int nelx, int nely) {
  const int nelxy = nelx * nely;
  *ez = 1 + (eg - 1) / nelxy;
  *ey = 1 + (mod1(eg, nelxy) - 1) / nelx;
  *ex = mod1(eg, nelx);
}

// set_vert_box, prox_dssum.f:42-73: lexicographic numbering of the GLL
// points of a nelx x nely x nelz box.
void set_vert_box(int64_t *glo_num, int nx, int nelt, int nelx, int nely,
                  const int *lglel) {
  const int nn = nx - 1;
  const int64_t ax = int64_t(nn) * nelx + 1, ay = int64_t(nn) * nely + 1;
  const int64_t nxyz = int64_t(nx) * nx * nx;
  for (int e = 0; e < nelt; ++e) {
    int ex, ey, ez;
    get_exyz(&ex, &ey, &ez, lglel[e], nelx, nely);
    int64_t *g = glo_num + nxyz * e;
    for (int k = 0; k <= nn; ++k)
      for (int j = 0; j <= nn; ++j)
        for (int i = 0; i <= nn; ++i) {
          const int64_t kg = int64_t(nn) * (ez - 1) + k;
          const int64_t jg = int64_t(nn) * (ey - 1) + j;
          const int64_t ig = int64_t(nn) * (ex - 1) + i;
          g[i + nx * j + int64_t(nx) * nx * k] = 1 + ig + jg * ax + kg * ax * ay;
        }
  }
}

// The domain-boundary faces of global element eg that get_face (cg.f:302-368)
// and get_bcs (hsmg.f:605-642) zero.
unsigned face_bits(int eg, int nelx, int nely, int nelz) {
  const int nelxy = nelx * nely;
  const int ir = 1 + (eg - 1) / nelxy;
  const int iq = 1 + (mod1(eg, nelxy) - 1) / nelx;
  const int ip = mod1(eg, nelx);
  unsigned f = 0;
  if (ip % nelx == 1 || nelx == 1) f |= 1u;
  if (ip % nelx == 0) f |= 2u;
  if (iq % nely == 1 || nely == 1) f |= 4u;
  if (iq % nely == 0) f |= 8u;
  if (ir % nelz == 1 || nelz == 1) f |= 16u;
  if (ir % nelz == 0) f |= 32u;
  return f;
}

// A x = lam B x, B symmetric positive definite: B-orthonormal eigenvectors
// (columns of a, overwritten) and ascending eigenvalues -- the contract of
// LAPACK dsygv(itype=1,'V','U') used by generalev (hsmg.f:483-523).  Method:
// Cholesky B = L L^T, cyclic Jacobi rotations on L^-1 A L^-T, X = L^-T Q.
int generalev(double *a, double *b, double *lam, int n) {
  std::vector<double> L(n * n, 0.), C(n * n, 0.), Q(n * n, 0.), T(n * n, 0.);
  auto at = [n](std::vector<double> &M, int i, int j) -> double & {
    return M[i + j * n];
  };
  for (int j = 0; j < n; ++j) {
    double s = b[j + j * n];
    for (int k = 0; k < j; ++k) s -= at(L, j, k) * at(L, j, k);
    if (!(s > 0)) return j + 1;
    at(L, j, j) = std::sqrt(s);
    for (int i = j + 1; i < n; ++i) {
      double t = b[i + j * n];
      for (int k = 0; k < j; ++k) t -= at(L, i, k) * at(L, j, k);
      at(L, i, j) = t / at(L, j, j);
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double t = a[i + j * n];
      for (int k = 0; k < i; ++k) t -= at(L, i, k) * at(T, k, j);
      at(T, i, j) = t / at(L, i, i);
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double t = at(T, j, i);
      for (int k = 0; k < i; ++k) t -= at(L, i, k) * at(C, j, k);
      at(C, j, i) = t / at(L, i, i);
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < j; ++i) {
      const double s = 0.5 * (at(C, i, j) + at(C, j, i));
      at(C, i, j) = s;
      at(C, j, i) = s;
    }
  for (int i = 0; i < n; ++i) at(Q, i, i) = 1.;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0., tot = 0.;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double v = at(C, i, j) * at(C, i, j);
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-34 * (tot > 0 ? tot : 1.)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = at(C, p, q);
        if (apq == 0.) continue;
        const double th = (at(C, q, q) - at(C, p, p)) / (2. * apq);
        const double t =
            (th >= 0 ? 1. : -1.) / (std::fabs(th) + std::sqrt(th * th + 1.));
        const double cs = 1. / std::sqrt(t * t + 1.), sn = t * cs;
        for (int k = 0; k < n; ++k) {
          const double x = at(C, k, p), y = at(C, k, q);
          at(C, k, p) = cs * x - sn * y;
          at(C, k, q) = sn * x + cs * y;
        }
        for (int k = 0; k < n; ++k) {
          const double x = at(C, p, k), y = at(C, q, k);
          at(C, p, k) = cs * x - sn * y;
          at(C, q, k) = sn * x + cs * y;
        }
        for (int k = 0; k < n; ++k) {
          const double x = at(Q, k, p), y = at(Q, k, q);
          at(Q, k, p) = cs * x - sn * y;
          at(Q, k, q) = sn * x + cs * y;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int x, int y) { return at(C, x, x) < at(C, y, y); });
  for (int jj = 0; jj < n; ++jj) {
    const int j = ord[jj];
    lam[jj] = at(C, j, j);
    for (int i = n - 1; i >= 0; --i) {
      double t = at(Q, i, j);
      for (int k = i + 1; k < n; ++k) t -= at(L, k, i) * a[k + jj * n];
      a[i + jj * n] = t / at(L, i, i);
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// jl local topology.  Semantics of nonzero_ids (gs.c:88-113): entries with a
// nonzero id are grouped by |id|; inside a group unflagged (positive) entries
// come before flagged (negative) ones, each in ascending local index; the
// first entry is the primary; groups are ordered by ascending primary.
// local_map (gs.c:330-357) then writes [primary, others..., -1]... -1,
// leaving out groups with no other member (and, for the unflagged map,
// flagged members).  Here: one LSD radix sort by |id| (stable, so local
// index order survives), a stable flag partition per group, and a bucket
// placement by primary.
void gs_topology(const int64_t *ids, int n, GsHost *out) {
  std::vector<uint32_t> idx;
  idx.reserve(n);
  uint64_t maxid = 0;
  for (int i = 0; i < n; ++i)
    if (ids[i] != 0) {
      idx.push_back(uint32_t(i));
      const uint64_t a = uint64_t(ids[i] < 0 ? -ids[i] : ids[i]);
      maxid = std::max(maxid, a);
    }
  const size_t m = idx.size();
  auto key = [&](uint32_t i) {
    return uint64_t(ids[i] < 0 ? -ids[i] : ids[i]);
  };
  std::vector<uint32_t> tmp(m);
  int bits = 0;
  while (bits < 64 && (maxid >> bits) != 0) bits += 11;
  for (int shift = 0; shift < bits; shift += 11) {
    std::vector<size_t> cnt(2049, 0);
    for (size_t q = 0; q < m; ++q) ++cnt[((key(idx[q]) >> shift) & 2047) + 1];
    for (int b = 0; b < 2048; ++b) cnt[b + 1] += cnt[b];
    for (size_t q = 0; q < m; ++q) tmp[cnt[(key(idx[q]) >> shift) & 2047]++] = idx[q];
    idx.swap(tmp);
  }
  // group boundaries; stable partition by flag; primary = first member
  std::vector<size_t> gstart;
  for (size_t q = 0; q < m; ++q)
    if (q == 0 || key(idx[q]) != key(idx[q - 1])) gstart.push_back(q);
  gstart.push_back(m);
  const size_t ngrp = gstart.size() - 1;
  for (size_t g = 0; g < ngrp; ++g)
    std::stable_partition(idx.begin() + gstart[g], idx.begin() + gstart[g + 1],
                          [&](uint32_t i) { return ids[i] > 0; });
  // order groups by primary (primaries are distinct local indices)
  std::vector<int64_t> by_primary(n, -1);
  for (size_t g = 0; g < ngrp; ++g) by_primary[idx[gstart[g]]] = int64_t(g);
  const uint32_t END = uint32_t(-1);
  for (int k = 0; k < 3; ++k) out->map[k].clear();
  for (int pr = 0; pr < n; ++pr) {
    const int64_t g = by_primary[pr];
    if (g < 0) continue;
    const size_t b = gstart[g], e = gstart[g + 1];
    const bool pflag = ids[idx[b]] < 0;
    // unflagged map: the primary, then following members while unflagged
    {
      size_t q = b + 1;
      while (q < e && ids[idx[q]] > 0) ++q;
      if (q > b + 1) {
        out->map[0].push_back(idx[b]);
        for (size_t r = b + 1; r < q; ++r) out->map[0].push_back(idx[r]);
        out->map[0].push_back(END);
      }
    }
    if (e > b + 1) {
      for (size_t r = b; r < e; ++r) out->map[1].push_back(idx[r]);
      out->map[1].push_back(END);
    }
    if (pflag) out->map[2].push_back(idx[b]);
  }
  for (int k = 0; k < 3; ++k) out->map[k].push_back(END);
}

}  // namespace nb

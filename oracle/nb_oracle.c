/*
 * nb_oracle.c -- CPU restatement of the Nekbone spectral-element Poisson CG
 * hot path (FP64).  See nb_oracle.h for the parity status of each part.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  Never linked into, loaded by or called from the product.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).  Floating-point contraction is controlled
 * explicitly: the library is built with -ffp-contract=off and, when
 * ORC_FMA=1, the multiply-add chains of the hot path are written as fma()
 * calls (the contraction gfortran applies on aarch64); with ORC_FMA=0 they are
 * separate multiply and add (gfortran's x86-64 default).
 */
#include "nb_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORC_FMA
#define ORC_FMA 0
#endif

#if ORC_FMA
#define MADD(acc, a, b) ((acc) = fma((a), (b), (acc)))
#define FMAC(a, b, c) fma((a), (b), (c)) /* a*b + c */
#else
#define MADD(acc, a, b) ((acc) = (acc) + (a) * (b))
#define FMAC(a, b, c) ((a) * (b) + (c))
#endif

int orc_fma_variant(void) { return ORC_FMA; }

#define NMAX 84

/* ======================================================================== */
/* speclib.f                                                                */
/* ======================================================================== */

/* GAMMAF, speclib.f:371-393 */
static double orc_gammaf(double x) {
  const double zero = 0.0, half = 0.5, one = 1.0, two = 2.0, four = 4.0;
  (void)zero;
  double pi = four * atan(one);
  double g = one;
  if (x == -half) g = -two * sqrt(pi);
  if (x == half) g = sqrt(pi);
  if (x == one) g = one;
  if (x == two) g = one;
  if (x == 1.5) g = sqrt(pi) / 2.;
  if (x == 2.5) g = 1.5 * sqrt(pi) / 2.;
  if (x == 3.5) g = 0.5 * (2.5 * (1.5 * sqrt(pi)));
  if (x == 3.) g = 2.;
  if (x == 4.) g = 6.;
  if (x == 5.) g = 24.;
  if (x == 6.) g = 120.;
  return g;
}

/* PNORMJ, speclib.f:395-419 */
static double pnormj(int n, double alpha, double beta) {
  const double one = 1., two = 2.;
  double dn = (double)n;
  double cnst = alpha + beta + one;
  double prod;
  if (n <= 1) {
    prod = orc_gammaf(dn + alpha) * orc_gammaf(dn + beta);
    prod = prod / (orc_gammaf(dn) * orc_gammaf(dn + alpha + beta));
    return prod * pow(two, cnst) / (two * dn + cnst);
  }
  prod = orc_gammaf(alpha + one) * orc_gammaf(beta + one);
  prod = prod / (two * (one + cnst) * orc_gammaf(cnst + one));
  prod = prod * (one + alpha) * (two + alpha);
  prod = prod * (one + beta) * (two + beta);
  for (int i = 3; i <= n; ++i) {
    double dindx = (double)i;
    double frac = (dindx + alpha) * (dindx + beta) /
                  (dindx * (dindx + alpha + beta));
    prod = prod * frac;
  }
  return prod * pow(two, cnst) / (two * dn + cnst);
}

/* JACOBF, speclib.f:479-518 */
static void jacobf(double *poly, double *pder, double *polym1, double *pderm1,
                   double *polym2, double *pderm2, int n, double alp,
                   double bet, double x) {
  double apb = alp + bet;
  double polyl, pderl, psave = 0., pdsave = 0.;
  *poly = 1.;
  *pder = 0.;
  if (n == 0) return;
  polyl = *poly;
  pderl = *pder;
  *poly = (alp - bet + (apb + 2.) * x) / 2.;
  *pder = (apb + 2.) / 2.;
  if (n == 1) return;
  for (int k = 2; k <= n; ++k) {
    double dk = (double)k;
    double a1 = 2. * dk * (dk + apb) * (2. * dk + apb - 2.);
    double a2 = (2. * dk + apb - 1.) * (alp * alp - bet * bet);
    double b3 = (2. * dk + apb - 2.);
    double a3 = b3 * (b3 + 1.) * (b3 + 2.);
    double a4 = 2. * (dk + alp - 1.) * (dk + bet - 1.) * (2. * dk + apb);
    double polyn = ((a2 + a3 * x) * *poly - a4 * polyl) / a1;
    double pdern = ((a2 + a3 * x) * *pder - a4 * pderl + a3 * *poly) / a1;
    psave = polyl;
    pdsave = pderl;
    polyl = *poly;
    *poly = polyn;
    pderl = *pder;
    *pder = pdern;
  }
  *polym1 = polyl;
  *pderm1 = pderl;
  *polym2 = psave;
  *pderm2 = pdsave;
}

/* JACG, speclib.f:421-477 (Newton with deflation, EPS=1e-12, KSTOP=10) */
static void jacg(double *xjac, int np, double alpha, double beta) {
  const int kstop = 10;
  const double eps = 1.0e-12;
  int n = np - 1;
  double one = 1.;
  double dth = 4. * atan(one) / (2. * ((double)n) + 2.);
  double xlast = 0.;
  for (int j = 1; j <= np; ++j) {
    double x;
    if (j == 1) {
      x = cos((2. * (((double)j) - 1.) + 1.) * dth);
    } else {
      double x1 = cos((2. * (((double)j) - 1.) + 1.) * dth);
      double x2 = xlast;
      x = (x1 + x2) / 2.;
    }
    for (int k = 1; k <= kstop; ++k) {
      double p, pd, pm1, pdm1, pm2, pdm2;
      jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np, alpha, beta, x);
      double recsum = 0.;
      for (int i = 1; i <= j - 1; ++i) recsum = recsum + 1. / (x - xjac[np - i]);
      double delx = -p / (pd - recsum * p);
      x = x + delx;
      if (fabs(delx) < eps) break;
    }
    xjac[np - j] = x;
    xlast = x;
  }
  for (int i = 1; i <= np; ++i) {
    double xmin = 2.;
    int jmin = i;
    for (int j = i; j <= np; ++j) {
      if (xjac[j - 1] < xmin) {
        xmin = xjac[j - 1];
        jmin = j;
      }
    }
    if (jmin != i) {
      double swap = xjac[i - 1];
      xjac[i - 1] = xjac[jmin - 1];
      xjac[jmin - 1] = swap;
    }
  }
}

/* ZWGJD, speclib.f:155-205 */
static void zwgjd(double *z, double *w, int np, double alpha, double beta) {
  const double one = 1., two = 2.;
  int n = np - 1;
  double apb = alpha + beta;
  if (np == 1) {
    z[0] = (beta - alpha) / (apb + two);
    w[0] = orc_gammaf(alpha + one) * orc_gammaf(beta + one) / orc_gammaf(apb + two) *
           pow(two, apb + one);
    return;
  }
  jacg(z, np, alpha, beta);
  int np1 = n + 1, np2 = n + 2;
  double dnp1 = (double)np1, dnp2 = (double)np2;
  double fac1 = dnp1 + alpha + beta + one;
  double fac2 = fac1 + dnp1;
  double fac3 = fac2 + one;
  double fnorm = pnormj(np1, alpha, beta);
  double rcoef = (fnorm * fac2 * fac3) / (two * fac1 * dnp2);
  for (int i = 0; i < np; ++i) {
    double p, pd, pm1, pdm1, pm2, pdm2;
    jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np2, alpha, beta, z[i]);
    w[i] = -rcoef / (p * pdm1);
  }
}

/* ENDW1, speclib.f:283-325 */
static double endw1(int n, double alpha, double beta) {
  const double zero = 0., one = 1., two = 2., three = 3., four = 4.;
  double apb = alpha + beta;
  if (n == 0) return zero;
  double f1 = orc_gammaf(alpha + two) * orc_gammaf(beta + one) / orc_gammaf(apb + three);
  f1 = f1 * (apb + two) * pow(two, apb + two) / two;
  if (n == 1) return f1;
  double fint1 = orc_gammaf(alpha + two) * orc_gammaf(beta + one) / orc_gammaf(apb + three);
  fint1 = fint1 * pow(two, apb + two);
  double fint2 = orc_gammaf(alpha + two) * orc_gammaf(beta + two) / orc_gammaf(apb + four);
  fint2 = fint2 * pow(two, apb + three);
  double f2 = (-two * (beta + two) * fint1 + (apb + four) * fint2) *
              (apb + three) / four;
  if (n == 2) return f2;
  double f3 = 0.;
  for (int i = 3; i <= n; ++i) {
    double di = (double)(i - 1);
    double abn = alpha + beta + di;
    double abnn = abn + di;
    double a1 = -(two * (di + alpha) * (di + beta)) / (abn * abnn * (abnn + one));
    double a2 = (two * (alpha - beta)) / (abnn * (abnn + two));
    double a3 = (two * (abn + one)) / ((abnn + two) * (abnn + one));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

/* ENDW2, speclib.f:327-369 */
static double endw2(int n, double alpha, double beta) {
  const double zero = 0., one = 1., two = 2., three = 3., four = 4.;
  double apb = alpha + beta;
  if (n == 0) return zero;
  double f1 = orc_gammaf(alpha + one) * orc_gammaf(beta + two) / orc_gammaf(apb + three);
  f1 = f1 * (apb + two) * pow(two, apb + two) / two;
  if (n == 1) return f1;
  double fint1 = orc_gammaf(alpha + one) * orc_gammaf(beta + two) / orc_gammaf(apb + three);
  fint1 = fint1 * pow(two, apb + two);
  double fint2 = orc_gammaf(alpha + two) * orc_gammaf(beta + two) / orc_gammaf(apb + four);
  fint2 = fint2 * pow(two, apb + three);
  double f2 = (two * (alpha + two) * fint1 - (apb + four) * fint2) *
              (apb + three) / four;
  if (n == 2) return f2;
  double f3 = 0.;
  for (int i = 3; i <= n; ++i) {
    double di = (double)(i - 1);
    double abn = alpha + beta + di;
    double abnn = abn + di;
    double a1 = -(two * (di + alpha) * (di + beta)) / (abn * abnn * (abnn + one));
    double a2 = (two * (alpha - beta)) / (abnn * (abnn + two));
    double a3 = (two * (abn + one)) / ((abnn + two) * (abnn + one));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

/* ZWGLJD, speclib.f:238-281 */
void orc_zwgljd(double *z, double *w, int np, double alpha, double beta) {
  const double one = 1., two = 2.;
  int n = np - 1, nm1 = n - 1;
  if (np <= 1) {
    fprintf(stderr, "ZWGLJD: Minimum number of Gauss-Lobatto points is 2\n");
    return;
  }
  if (nm1 > 0) zwgjd(z + 1, w + 1, nm1, alpha + one, beta + one);
  z[0] = -one;
  z[np - 1] = one;
  for (int i = 2; i <= np - 1; ++i) w[i - 1] = w[i - 1] / (one - z[i - 1] * z[i - 1]);
  double p, pd, pm1, pdm1, pm2, pdm2;
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[0]);
  w[0] = endw1(n, alpha, beta) / (two * pd);
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[np - 1]);
  w[np - 1] = endw2(n, alpha, beta) / (two * pd);
}

/* ZWGLL, speclib.f:107-122 (ZWGLJ speclib.f:207-236 copies through) */
void orc_zwgll(double *z, double *w, int np) { orc_zwgljd(z, w, np, 0., 0.); }

/* fd_weights_full, semhat.f:39-93 (Fornberg); c is (0:n, 0:m) column-major */
void orc_fd_weights_full(double xx, const double *x, int n, int m, double *c) {
#define C_(j, k) c[(j) + (k) * (n + 1)]
  double c1 = 1.;
  double c4 = x[0] - xx;
  for (int k = 0; k <= m; ++k)
    for (int j = 0; j <= n; ++j) C_(j, k) = 0.;
  C_(0, 0) = 1.;
  for (int i = 1; i <= n; ++i) {
    int mn = i < m ? i : m;
    double c2 = 1.;
    double c5 = c4;
    c4 = x[i] - xx;
    for (int j = 0; j <= i - 1; ++j) {
      double c3 = x[i] - x[j];
      c2 = c2 * c3;
      for (int k = mn; k >= 1; --k)
        C_(i, k) = c1 * (k * C_(i - 1, k - 1) - c5 * C_(i - 1, k)) / c2;
      C_(i, 0) = -c1 * c5 * C_(i - 1, 0) / c2;
      for (int k = mn; k >= 1; --k)
        C_(j, k) = (c4 * C_(j, k) - k * C_(j, k - 1)) / c3;
      C_(j, 0) = c4 * C_(j, 0) / c3;
    }
    c1 = c2;
  }
#undef C_
}

/* semhat, semhat.f:2-37.  a,c,d are (0:n,0:n) column-major. */
void orc_semhat(double *a, double *b, double *c, double *d, double *z, int n) {
  int np = n + 1;
  double w[2 * NMAX + 2];
  orc_zwgll(z, b, np);
  for (int i = 0; i <= n; ++i) {
    orc_fd_weights_full(z[i], z, n, 1, w);
    for (int j = 0; j <= n; ++j) d[i + j * np] = w[j + np];
  }
  for (int i = 0; i < np * np; ++i) a[i] = 0.;
  for (int j = 0; j <= n; ++j)
    for (int i = 0; i <= n; ++i) {
      for (int k = 0; k <= n; ++k)
        a[i + j * np] = a[i + j * np] + d[k + i * np] * b[k] * d[k + j * np];
      c[i + j * np] = b[i] * d[i + j * np];
    }
}

/* ======================================================================== */
/* driver.f / prox_dssum.f                                                  */
/* ======================================================================== */

/* mod1, math.f:418-433 */
static int mod1(int i, int n) {
  if (i == 0) return 0;
  if (n == 0) return 0;
  int ii = i + n - 1;
  return ii % n + 1;
}

/* cubic, driver.f:196-247 */
void orc_cubic(int *mx, int *my, int *mz, int np) {
  *mx = np;
  *my = 1;
  *mz = 1;
  double ratio = np;
  int iroot3 = (int)(pow((double)np, 1. / 3.) + 0.000001);
  for (int i = iroot3; i >= 1; --i) {
    int iz = i, ix = 0, iy = 0;
    int myx = np / iz;
    int nrem = np - myx * iz;
    if (nrem == 0) {
      int iroot2 = (int)(pow((double)myx, 1. / 2.) + 0.000001);
      for (int j = iroot2; j >= 1; --j) {
        iy = j;
        ix = myx / iy;
        nrem = myx - ix * iy;
        if (nrem == 0) break;
      }
      int it;
      if (ix < iy) { it = ix; ix = iy; iy = it; }
      if (ix < iz) { it = ix; ix = iz; iz = it; }
      if (iy < iz) { it = iy; iy = iz; iz = it; }
      if ((double)ix / iz < ratio) {
        ratio = (double)ix / iz;
        *mx = ix;
        *my = iy;
        *mz = iz;
      }
    }
  }
}

/* init_mesh, driver.f:117-194, for a single process (np=1, nid=0). */
void orc_init_mesh(int ifbrick, int nelt, int mx, int my, int mz, int *nelx,
                   int *nely, int *nelz, int *lglel) {
  const int np = 1, nid = 0;
  int npx = 0, npy = 0, npz = 0;
  if (!ifbrick) {
    *nelx = nelt * np;
    *nely = 1;
    *nelz = 1;
    for (int e = 1; e <= nelt; ++e) lglel[e - 1] = e + nid * nelt;
    return;
  }
  if (npx * npy * npz != np) orc_cubic(&npx, &npy, &npz, np);
  if (mx * my * mz != nelt) orc_cubic(&mx, &my, &mz, nelt);
  *nelx = mx * npx;
  *nely = my * npy;
  *nelz = mz * npz;
  int offs = ((nid % npx) * mx) + npx * (my * mx) * ((nid / npx) % npy) +
             (npx * npy) * (mx * my * mz) * (nid / (npx * npy));
  int e = 0;
  for (int k = 0; k < mz; ++k)
    for (int j = 0; j < my; ++j)
      for (int i = 0; i < mx; ++i)
        lglel[e++] = offs + i + (j * *nelx) + (k * *nelx * *nely) + 1;
}

/* get_exyz, prox_dssum.f:75-86 */
static void get_exyz(int *ex, int *ey, int *ez, int eg, int nelx, int nely) {
  int nelxy = nelx * nely;
  *ez = 1 + (eg - 1) / nelxy;
  *ey = mod1(eg, nelxy);
  *ey = 1 + (*ey - 1) / nelx;
  *ex = mod1(eg, nelx);
}

/* set_vert_box, prox_dssum.f:42-73 */
void orc_set_vert_box(int64_t *glo_num, int nx, int nelt, int nelx, int nely,
                      int nelz, const int *lglel) {
  (void)nelz;
  int nn = nx - 1;
  for (int e = 1; e <= nelt; ++e) {
    int ex, ey, ez;
    get_exyz(&ex, &ey, &ez, lglel[e - 1], nelx, nely);
    for (int k = 0; k <= nn; ++k)
      for (int j = 0; j <= nn; ++j)
        for (int i = 0; i <= nn; ++i) {
          int64_t kg = (int64_t)nn * (ez - 1) + k;
          int64_t jg = (int64_t)nn * (ey - 1) + j;
          int64_t ig = (int64_t)nn * (ex - 1) + i;
          int32_t ax = nn * nelx + 1, ay = nn * nely + 1;
          int64_t ii = 1 + ig + jg * ax + kg * ax * ay;
          int64_t ll = 1 + i + (int64_t)nx * j + (int64_t)nx * nx * k +
                       (int64_t)nx * nx * nx * (e - 1);
          glo_num[ll - 1] = ii;
        }
  }
}

/* ======================================================================== */
/* jl gather-scatter (src/jl/gs.c, src/jl/gs_local.c), single process       */
/* ======================================================================== */

typedef struct {
  uint64_t id;
  uint32_t i, flag, primary;
} nz_row;

struct orc_gs {
  uint32_t *map[3]; /* 0 unflagged, 1 all, 2 flagged primaries */
  int len[3];
};

static int cmp_id_flag_i(const void *pa, const void *pb) {
  const nz_row *a = pa, *b = pb;
  if (a->id != b->id) return a->id < b->id ? -1 : 1;
  if (a->flag != b->flag) return a->flag < b->flag ? -1 : 1;
  if (a->i != b->i) return a->i < b->i ? -1 : 1;
  return 0;
}
static int cmp_primary_flag_i(const void *pa, const void *pb) {
  const nz_row *a = pa, *b = pb;
  if (a->primary != b->primary) return a->primary < b->primary ? -1 : 1;
  if (a->flag != b->flag) return a->flag < b->flag ? -1 : 1;
  if (a->i != b->i) return a->i < b->i ? -1 : 1;
  return 0;
}

/* local_map, gs.c:330-357.  nz sorted by primary, then flag, then index. */
static uint32_t *local_map(const nz_row *nz, int n, int ignore_flagged,
                           int *len) {
  const uint32_t END = (uint32_t)-1;
  long count = 1;
  for (int row = 0; row < n;) {
    uint64_t id = nz[row].id;
    int any = 0, other;
    for (other = row + 1; other < n && nz[other].id == id &&
                          (!ignore_flagged || nz[other].flag == 0);
         ++other)
      any = 2, ++count;
    count += any;
    row = other;
  }
  uint32_t *map = malloc(sizeof(uint32_t) * count), *p = map;
  for (int row = 0; row < n;) {
    uint64_t id = nz[row].id;
    int any = 0, other;
    *p++ = nz[row].i;
    for (other = row + 1; other < n && nz[other].id == id &&
                          (!ignore_flagged || nz[other].flag == 0);
         ++other)
      any = 1, *p++ = nz[other].i;
    if (any)
      *p++ = END;
    else
      --p;
    row = other;
  }
  *p++ = END;
  *len = (int)(p - map);
  return map;
}

/* nonzero_ids gs.c:88-113 + local_setup gs.c:1064-1069 +
 * flagged_primaries_map gs.c:359-370.  At one process the remote part of the
 * topology is empty. */
orc_gs *orc_gs_setup(const int64_t *ids, int n) {
  nz_row *nz = malloc(sizeof(nz_row) * (n > 0 ? n : 1));
  int m = 0;
  for (int i = 0; i < n; ++i) {
    int64_t id = ids[i];
    if (id == 0) continue;
    uint64_t aid = (uint64_t)(id < 0 ? -id : id);
    nz[m].id = aid;
    nz[m].i = (uint32_t)i;
    nz[m].flag = id < 0;
    nz[m].primary = 0;
    ++m;
  }
  qsort(nz, m, sizeof(nz_row), cmp_id_flag_i);
  uint64_t last = (uint64_t)-1;
  uint32_t primary = (uint32_t)-1;
  for (int r = 0; r < m; ++r) {
    if (nz[r].id != last) primary = nz[r].i;
    nz[r].primary = primary;
    last = nz[r].id;
  }
  qsort(nz, m, sizeof(nz_row), cmp_primary_flag_i);
  orc_gs *h = calloc(1, sizeof(orc_gs));
  h->map[0] = local_map(nz, m, 1, &h->len[0]);
  h->map[1] = local_map(nz, m, 0, &h->len[1]);
  int cnt = 1;
  for (int r = 0; r < m; ++r)
    if (nz[r].i == nz[r].primary && nz[r].flag == 1) ++cnt;
  h->map[2] = malloc(sizeof(uint32_t) * cnt);
  int q = 0;
  for (int r = 0; r < m; ++r)
    if (nz[r].i == nz[r].primary && nz[r].flag == 1) h->map[2][q++] = nz[r].i;
  h->map[2][q++] = (uint32_t)-1;
  h->len[2] = q;
  free(nz);
  return h;
}

void orc_gs_free(orc_gs *h) {
  if (!h) return;
  for (int k = 0; k < 3; ++k) free(h->map[k]);
  free(h);
}

int orc_gs_map_len(const orc_gs *h, int which) { return h->len[which]; }
void orc_gs_map_copy(const orc_gs *h, int which, uint32_t *out) {
  memcpy(out, h->map[which], sizeof(uint32_t) * h->len[which]);
}

/* gather_T_OP / scatter_T / init_T, gs_local.c:60-97; gs_aux gs.c:1029-1045 */
#define GS_KERNELS(T, SUF, MINV, MAXV)                                         \
  static void gather_##SUF(T *u, const uint32_t *map, int op) {                \
    const uint32_t END = (uint32_t)-1;                                         \
    uint32_t i, j;                                                             \
    while ((i = *map++) != END) {                                              \
      T t = u[i];                                                              \
      j = *map++;                                                              \
      do {                                                                     \
        T q = u[j];                                                            \
        switch (op) {                                                          \
          case 1: t += q; break;                                               \
          case 2: t *= q; break;                                               \
          case 3: if (q < t) t = q; break;                                     \
          default: if (q > t) t = q; break;                                    \
        }                                                                      \
      } while ((j = *map++) != END);                                           \
      u[i] = t;                                                                \
    }                                                                          \
  }                                                                            \
  static void scatter_##SUF(T *u, const uint32_t *map) {                       \
    const uint32_t END = (uint32_t)-1;                                         \
    uint32_t i, j;                                                             \
    while ((i = *map++) != END) {                                              \
      T t = u[i];                                                              \
      j = *map++;                                                              \
      do u[j] = t;                                                             \
      while ((j = *map++) != END);                                             \
    }                                                                          \
  }                                                                            \
  static void init_##SUF(T *u, const uint32_t *map, int op) {                  \
    const uint32_t END = (uint32_t)-1;                                         \
    static const T ident[4] = {(T)0, (T)1, MAXV, MINV};                        \
    uint32_t i;                                                                \
    while ((i = *map++) != END) u[i] = ident[op - 1];                          \
  }

GS_KERNELS(double, d, -DBL_MAX, DBL_MAX)
GS_KERNELS(float, f, -FLT_MAX, FLT_MAX)
GS_KERNELS(int, i, INT_MIN, INT_MAX)
GS_KERNELS(int64_t, l, INT64_MIN, INT64_MAX)

void orc_gs_op(const orc_gs *h, void *u, int dom, int op, int transpose) {
  const uint32_t *mg = h->map[transpose ? 1 : 0];
  const uint32_t *ms = h->map[transpose ? 0 : 1];
  switch (dom) {
    case 1:
      gather_d(u, mg, op);
      if (!transpose) init_d(u, h->map[2], op);
      scatter_d(u, ms);
      break;
    case 2:
      gather_f(u, mg, op);
      if (!transpose) init_f(u, h->map[2], op);
      scatter_f(u, ms);
      break;
    case 3:
      gather_i(u, mg, op);
      if (!transpose) init_i(u, h->map[2], op);
      scatter_i(u, ms);
      break;
    default:
      gather_l(u, mg, op);
      if (!transpose) init_l(u, h->map[2], op);
      scatter_l(u, ms);
      break;
  }
}

/* ======================================================================== */
/* solver context (common blocks /dimn/ /dxyz/ /mymask/ /cflops/ ...)        */
/* ======================================================================== */

typedef struct {
  int nlev;
  int nx[8], nh[8];       /* 1-based levels */
  double *ah[8], *bh[8], *dh[8], *zh[8];
  double *jh[8], *jht[8]; /* level l: nh[l+1] x nh[l] */
  orc_gs *gsh[8], *gsh_schwarz[8];
  double *rstr_wt[8];    /* (nh, nh, 2, 3, nelt) */
  double *fast_s[8];     /* (nl*nl, 2, 3, nelt) */
  double *fast_d[8];     /* (nl^3, nelt) */
  double *schwarz_wt[8]; /* (nh, nh, 4, 3, nelt) */
  int *mask[8];          /* h1mg_setup_mask layout, 1-based content */
  int ntot[8];
  double *work, *work2;  /* extended arrays, 2 * nl^3 * nelt */
  double *e, *w, *r;     /* /scrmg/ */
  int ready;
} orc_mg;

struct orc_ctx {
  int nelx, nely, nelz, nelt, nx1, nxyz, n;
  int *lglel;
  int mask_mode, nthreads;
  double dxm1[NMAX * NMAX], dxtm1[NMAX * NMAX], wxm1[NMAX], zgm1[NMAX];
  orc_gs *gsh;
  double *cmask;   /* cmask[0] = pmask(-1), cmask[1] = pmask(0), ... */
  int *fullmask;   /* mask_mode 1: all boundary indices */
  int nfullmask;
  double flop_a, flop_cg;
  orc_mg mg;
};

int orc_ctx_n(const orc_ctx *c) { return c->n; }
const double *orc_ctx_dxm1(const orc_ctx *c) { return c->dxm1; }
const double *orc_ctx_wxm1(const orc_ctx *c) { return c->wxm1; }
const double *orc_ctx_zgm1(const orc_ctx *c) { return c->zgm1; }
double orc_flop_a(const orc_ctx *c) { return c->flop_a; }
double orc_flop_cg(const orc_ctx *c) { return c->flop_cg; }
void orc_ctx_reset_mask(orc_ctx *c) { c->cmask[0] = 1.0; }

/* int32 arithmetic with the wraparound the reference's default-integer
 * flop counters see (cg.f:81, cg.f:122). */
static int32_t i32mul(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a * (uint32_t)b);
}
static int32_t i32add(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a + (uint32_t)b);
}

/* masking, cg.f:269-284 */
static void masking(double *w, int nx, int e, int x0, int x1, int y0, int y1,
                    int z0, int z1) {
  long nxyz = (long)nx * nx * nx;
  for (int k = z0; k <= z1; ++k)
    for (int j = y0; j <= y1; ++j)
      for (int i = x0; i <= x1; ++i)
        w[(i - 1) + (long)nx * (j - 1) + (long)nx * nx * (k - 1) +
          nxyz * (e - 1)] = 0.0;
}

/* get_face, cg.f:302-368 */
static void get_face(const orc_ctx *c, double *w, int nx, int ie) {
  int x0 = 1, y0 = 1, z0 = 1, x1 = nx, y1 = nx, z1 = nx;
  int nelx = c->nelx, nely = c->nely, nelz = c->nelz;
  int nelxy = nelx * nely;
  int ngl = c->lglel[ie - 1];
  int ir = 1 + (ngl - 1) / nelxy;
  int iq = mod1(ngl, nelxy);
  iq = 1 + (iq - 1) / nelx;
  int ip = mod1(ngl, nelx);
  if (ip % nelx == 1 || nelx == 1) { x0 = 1; x1 = 1; masking(w, nx, ie, x0, x1, y0, y1, z0, z1); }
  if (ip % nelx == 0) { x0 = nx; x1 = nx; masking(w, nx, ie, x0, x1, y0, y1, z0, z1); }
  x0 = 1; x1 = nx;
  if (iq % nely == 1 || nely == 1) { y0 = 1; y1 = 1; masking(w, nx, ie, x0, x1, y0, y1, z0, z1); }
  if (iq % nely == 0) { y0 = nx; y1 = nx; masking(w, nx, ie, x0, x1, y0, y1, z0, z1); }
  y0 = 1; y1 = nx;
  if (ir % nelz == 1 || nelz == 1) { z0 = 1; z1 = 1; masking(w, nx, ie, x0, x1, y0, y1, z0, z1); }
  if (ir % nelz == 0) { z1 = nx; z0 = nx; masking(w, nx, ie, x0, x1, y0, y1, z0, z1); }
}

/* maskit, cg.f:214-258 with the pmask array of the caller (reference mode).
 * pmask[0] is pmask(-1), pmask[1] is pmask(0). */
static void maskit_ref(const orc_ctx *c, double *w, double *pmask, int nx) {
  int nxyz = nx * nx * nx;
  if (pmask[0] < 0) {
    int j = (int)pmask[1];
    for (int i = 1; i <= j; ++i) {
      int k = (int)pmask[1 + i];
      w[k - 1] = 0.0;
    }
  } else {
    int nn = 0;
    for (int e = 1; e <= c->nelt; ++e) {
      get_face(c, w, nx, e);
      for (int i = 1; i <= nxyz; ++i)
        if (w[i - 1] == 0) {
          nn = nn + 1;
          pmask[1 + nn] = i;
        }
    }
    pmask[0] = -1.;
    pmask[1] = nn;
  }
}

void orc_maskit(orc_ctx *c, double *w) {
  if (c->mask_mode == 0) {
    maskit_ref(c, w, c->cmask, c->nx1);
  } else {
    for (int q = 0; q < c->nfullmask; ++q) w[c->fullmask[q]] = 0.0;
  }
}

/* proxy_setup, prox_setup.f:2-25 (D, Dt, GLL points and weights) */
static void proxy_setup(orc_ctx *c) {
  int nx1 = c->nx1;
  double a[NMAX * NMAX], b[NMAX], cc[NMAX * NMAX], d[NMAX * NMAX], z[NMAX];
  orc_semhat(a, b, cc, d, z, nx1 - 1);
  for (int i = 0; i < nx1 * nx1; ++i) c->dxm1[i] = d[i];
  for (int j = 0; j < nx1; ++j)
    for (int i = 0; i < nx1; ++i) c->dxtm1[i + j * nx1] = d[j + i * nx1];
  for (int i = 0; i < nx1; ++i) {
    c->zgm1[i] = z[i];
    c->wxm1[i] = b[i];
  }
}

orc_ctx *orc_ctx_new(int nelx, int nely, int nelz, int nelt, int nx1,
                     const int *lglel, int mask_mode, int nthreads) {
  orc_ctx *c = calloc(1, sizeof(orc_ctx));
  c->nelx = nelx;
  c->nely = nely;
  c->nelz = nelz;
  c->nelt = nelt;
  c->nx1 = nx1;
  c->nxyz = nx1 * nx1 * nx1;
  c->n = c->nxyz * nelt;
  c->mask_mode = mask_mode;
  c->nthreads = nthreads > 0 ? nthreads : 1;
  c->lglel = malloc(sizeof(int) * nelt);
  memcpy(c->lglel, lglel, sizeof(int) * nelt);
  proxy_setup(c);
  /* proxy_setupds, prox_dssum.f:14-40 */
  int64_t *glo = malloc(sizeof(int64_t) * (size_t)c->n);
  orc_set_vert_box(glo, nx1, nelt, nelx, nely, nelz, c->lglel);
  c->gsh = orc_gs_setup(glo, c->n);
  free(glo);
  c->cmask = calloc((size_t)c->n + 2, sizeof(double));
  c->cmask[0] = 1.0; /* init_mesh, driver.f:125 */
  /* full Dirichlet mask: every element's outer faces (get_face per element) */
  double *t = malloc(sizeof(double) * (size_t)c->n);
  for (long i = 0; i < c->n; ++i) t[i] = 1.0;
  for (int e = 1; e <= nelt; ++e) get_face(c, t, nx1, e);
  int cnt = 0;
  for (long i = 0; i < c->n; ++i) cnt += t[i] == 0.0;
  c->fullmask = malloc(sizeof(int) * (cnt > 0 ? cnt : 1));
  c->nfullmask = cnt;
  cnt = 0;
  for (long i = 0; i < c->n; ++i)
    if (t[i] == 0.0) c->fullmask[cnt++] = (int)i;
  free(t);
  return c;
}

static void mg_free(orc_mg *m);

/* Threads of the OpenMP loops of later calls (1 = the scalar restatement). */
void orc_ctx_set_threads(orc_ctx *c, int nthreads) { c->nthreads = nthreads > 0 ? nthreads : 1; }

void orc_ctx_free(orc_ctx *c) {
  if (!c) return;
  orc_gs_free(c->gsh);
  mg_free(&c->mg);
  free(c->lglel);
  free(c->cmask);
  free(c->fullmask);
  free(c);
}

/* setup_g, prox_setup.f:27-52: g1=g4=g6=w_i w_j w_k, g2=g3=g5=0 */
void orc_setup_g(const orc_ctx *c, double *g) {
  int nx1 = c->nx1;
  long p = 0;
  for (int e = 0; e < c->nelt; ++e)
    for (int k = 0; k < nx1; ++k)
      for (int j = 0; j < nx1; ++j)
        for (int i = 0; i < nx1; ++i, ++p) {
          double *gp = g + 6 * p;
          for (int q = 0; q < 6; ++q) gp[q] = 0.;
          double v = c->wxm1[i] * c->wxm1[j] * c->wxm1[k];
          gp[0] = v;
          gp[3] = v;
          gp[5] = v;
        }
}

/* dssum, prox_dssum.f:2-12 */
void orc_dssum(orc_ctx *c, double *f) { orc_gs_op(c->gsh, f, 1, 1, 0); }

/* set_multiplicity, driver.f:274-291 */
void orc_set_multiplicity(orc_ctx *c, double *mult) {
  for (long i = 0; i < c->n; ++i) mult[i] = 1.0;
  orc_gs_op(c->gsh, mult, 1, 1, 0);
  for (long i = 0; i < c->n; ++i) mult[i] = 1. / mult[i];
}

/* set_f, driver.f:88-101 (i*i in default integer, wrapping) */
void orc_set_f(orc_ctx *c, double *f, const double *mult) {
  for (int i = 1; i <= c->n; ++i) {
    double arg = 1.e9 * (double)i32mul(i, i);
    arg = 1.e9 * cos(arg);
    f[i - 1] = sin(arg);
  }
  orc_dssum(c, f);
  for (long i = 0; i < c->n; ++i) f[i] = f[i] * mult[i];
}

/* ======================================================================== */
/* math.f / mxm                                                             */
/* ======================================================================== */

/* mxm -> mxmf2 -> mxfN, mxm_wrapper.f:1-52, mxm_std.f:1-66 (mxf12 :255):
 * c(i,j) = a(i,1)*b(1,j) + a(i,2)*b(2,j) + ... summed left to right.
 * mxm44_0 (n2>24, mxm_std.f:632) sums from 0 in the same order. */
void orc_mxm(const double *a, int n1, const double *b, int n2, double *c,
             int n3) {
  for (int j = 0; j < n3; ++j)
    for (int i = 0; i < n1; ++i) {
      double s = a[i] * b[j * n2];
      for (int k = 1; k < n2; ++k) MADD(s, a[i + (long)k * n1], b[k + (long)j * n2]);
      c[i + (long)j * n1] = s;
    }
}

/* glsc3, math.f:603-617 (sequential; gop is the identity at one process) */
double orc_glsc3(const double *a, const double *b, const double *mult, int n) {
  double tmp = 0.0;
  for (int i = 0; i < n; ++i) MADD(tmp, a[i] * b[i], mult[i]);
  return tmp;
}

/* parallel variant used only when nthreads > 1 (timing baseline): fixed
 * chunks summed in chunk order */
static double glsc3_ctx(const orc_ctx *c, const double *a, const double *b,
                        const double *mult, int n) {
  if (c->nthreads <= 1) return orc_glsc3(a, b, mult, n);
  double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : s) num_threads(c->nthreads) schedule(static)
#endif
  for (int i = 0; i < n; ++i) MADD(s, a[i] * b[i], mult[i]);
  return s;
}

/* add2s1, math.f:534-541: a = c1*a + b */
void orc_add2s1(double *a, const double *b, double c1, int n) {
  for (int i = 0; i < n; ++i) a[i] = FMAC(c1, a[i], b[i]);
}

/* add2s2, math.f:544-551: a = a + c1*b */
void orc_add2s2(double *a, const double *b, double c1, int n) {
  for (int i = 0; i < n; ++i) a[i] = FMAC(c1, b[i], a[i]);
}

/* ======================================================================== */
/* cg.f                                                                     */
/* ======================================================================== */

/* local_grad3, cg.f:170-187 */
void orc_local_grad3(double *ur, double *us, double *ut, const double *u,
                     int n, const double *D, const double *Dt) {
  int m1 = n + 1, m2 = m1 * m1;
  orc_mxm(D, m1, u, m1, ur, m2);
  for (int k = 0; k <= n; ++k)
    orc_mxm(u + (long)k * m2, m1, Dt, m1, us + (long)k * m2, m1);
  orc_mxm(u, m2, Dt, m1, ut, m1);
}

/* local_grad3_t, cg.f:189-212 */
void orc_local_grad3_t(double *u, const double *ur, const double *us,
                       const double *ut, int n, const double *D,
                       const double *Dt, double *w) {
  int m1 = n + 1, m2 = m1 * m1, m3 = m2 * m1;
  orc_mxm(Dt, m1, ur, m1, u, m2);
  for (int k = 0; k <= n; ++k)
    orc_mxm(us + (long)k * m2, m1, D, m1, w + (long)k * m2, m1);
  for (int i = 0; i < m3; ++i) u[i] = u[i] + w[i]; /* add2, math.f:504 */
  orc_mxm(ut, m2, D, m1, w, m1);
  for (int i = 0; i < m3; ++i) u[i] = u[i] + w[i];
}

/* ax_e, cg.f:142-168 with caller-provided scratch */
static void ax_e_scr(const orc_ctx *c, double *w, const double *u,
                     const double *g, double *ur, double *us, double *ut,
                     double *wk) {
  int nxyz = c->nxyz, n = c->nx1 - 1;
  orc_local_grad3(ur, us, ut, u, n, c->dxm1, c->dxtm1);
  for (int i = 0; i < nxyz; ++i) {
    const double *gi = g + 6 * (long)i;
    double wr = gi[0] * ur[i];
    MADD(wr, gi[1], us[i]);
    MADD(wr, gi[2], ut[i]);
    double ws = gi[1] * ur[i];
    MADD(ws, gi[3], us[i]);
    MADD(ws, gi[4], ut[i]);
    double wt = gi[2] * ur[i];
    MADD(wt, gi[4], us[i]);
    MADD(wt, gi[5], ut[i]);
    ur[i] = wr;
    us[i] = ws;
    ut[i] = wt;
  }
  orc_local_grad3_t(w, ur, us, ut, n, c->dxm1, c->dxtm1, wk);
}

void orc_ax_e(orc_ctx *c, double *w, const double *u, const double *g) {
  int nxyz = c->nxyz;
  double *scr = malloc(sizeof(double) * 4 * nxyz);
  ax_e_scr(c, w, u, g, scr, scr + nxyz, scr + 2 * nxyz, scr + 3 * nxyz);
  free(scr);
}

/* element loop of ax, cg.f:111-114 */
void orc_ax_local(orc_ctx *c, double *w, const double *u, const double *g) {
  int nxyz = c->nxyz, nelt = c->nelt;
#ifdef _OPENMP
#pragma omp parallel num_threads(c->nthreads)
#endif
  {
    double *scr = malloc(sizeof(double) * 4 * nxyz);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int e = 0; e < nelt; ++e)
      ax_e_scr(c, w + (long)e * nxyz, u + (long)e * nxyz,
               g + 6L * nxyz * e, scr, scr + nxyz, scr + 2 * nxyz,
               scr + 3 * nxyz);
    free(scr);
  }
}

/* ax, cg.f:96-125 */
void orc_ax(orc_ctx *c, double *w, const double *u, const double *g) {
  orc_ax_local(c, w, u, g);
  orc_dssum(c, w);
  orc_add2s2(w, u, .1, c->n);
  orc_maskit(c, w);
  int32_t nxyz = c->nxyz;
  int32_t fa = i32mul(i32add(i32mul(19, nxyz), i32mul(i32mul(12, c->nx1), nxyz)),
                      c->nelt);
  c->flop_a = c->flop_a + (double)fa;
}

/* cg, cg.f:2-84.  solveM (cg.f:86-94) is h1mg_solve (MGRID, hsmg.f:960) or
 * the copy of hsmg_dum.f:9-14. */
int orc_cg(orc_ctx *c, double *x, const double *f, const double *g,
           const double *mult, double *r, double *w, double *p, double *z,
           int n, int niter, int use_mg, double *hist) {
  double pap = 0.0, rtz1 = 1.0, rtz2, beta, alpha = 0.0, alphm, rtr, rnorm;
  double one = 1., eps = 1.e-20;
  if (one + eps == one) eps = 1.e-14;
  if (one + eps == one) eps = 1.e-7;
  (void)eps;
  for (int i = 0; i < n; ++i) x[i] = 0.0;
  memcpy(r, f, sizeof(double) * n);
  orc_maskit(c, r);
  rnorm = sqrt(glsc3_ctx(c, r, mult, r, n));
  if (hist) {
    hist[0] = rnorm;
    hist[1] = hist[2] = hist[3] = hist[4] = 0.;
  }
  beta = 0.0;
  int iter;
  for (iter = 1; iter <= niter; ++iter) {
    if (use_mg)
      orc_h1mg_solve(c, z, r, n);
    else
      memcpy(z, r, sizeof(double) * n);
    rtz2 = rtz1;
    rtz1 = glsc3_ctx(c, r, mult, z, n);
    beta = rtz1 / rtz2;
    if (iter == 1) beta = 0.0;
    orc_add2s1(p, z, beta, n);
    orc_ax(c, w, p, g);
    pap = glsc3_ctx(c, w, mult, p, n);
    alpha = rtz1 / pap;
    alphm = -alpha;
    orc_add2s2(x, p, alpha, n);
    orc_add2s2(r, w, alphm, n);
    rtr = glsc3_ctx(c, r, mult, r, n);
    rnorm = sqrt(rtr);
    if (hist) {
      double *hh = hist + 5 * iter;
      hh[0] = rnorm;
      hh[1] = alpha;
      hh[2] = beta;
      hh[3] = pap;
      hh[4] = rtz1;
    }
  }
  int32_t fc = i32mul(i32mul(iter, 15), n);
  c->flop_cg = c->flop_cg + (double)fc;
  return iter;
}

/* ======================================================================== */
/* hsmg.f                                                                   */
/* ======================================================================== */

/* Generalized symmetric-definite eigenproblem A x = lam B x with B-orthonormal
 * eigenvectors and ascending eigenvalues: the contract of LAPACK dsygv
 * (itype=1, jobz='V', uplo='U') that generalev (hsmg.f:483-523) relies on.
 * Restated from the mathematics: Cholesky B = L L^T, cyclic Jacobi on
 * L^-1 A L^-T, back-transform X = L^-T Q.  a (n x n, column-major) is
 * overwritten by X.  Returns 0 on success. */
int orc_generalev(double *a, double *b, double *lam, int n) {
  double *L = calloc((size_t)n * n, sizeof(double));
  double *C = calloc((size_t)n * n, sizeof(double));
  double *Q = calloc((size_t)n * n, sizeof(double));
  double *T = calloc((size_t)n * n, sizeof(double));
#define M_(X, i, j) X[(i) + (long)(j) * n]
  int info = 0;
  for (int j = 0; j < n && !info; ++j) {
    double s = M_(b, j, j);
    for (int k = 0; k < j; ++k) s -= M_(L, j, k) * M_(L, j, k);
    if (s <= 0) { info = j + 1; break; }
    M_(L, j, j) = sqrt(s);
    for (int i = j + 1; i < n; ++i) {
      double t = M_(b, i, j);
      for (int k = 0; k < j; ++k) t -= M_(L, i, k) * M_(L, j, k);
      M_(L, i, j) = t / M_(L, j, j);
    }
  }
  if (!info) {
    /* T = L^-1 A  (forward substitution, column by column) */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double t = M_(a, i, j);
        for (int k = 0; k < i; ++k) t -= M_(L, i, k) * M_(T, k, j);
        M_(T, i, j) = t / M_(L, i, i);
      }
    /* C = T L^-T = (L^-1 T^T)^T */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double t = M_(T, j, i);
        for (int k = 0; k < i; ++k) t -= M_(L, i, k) * M_(C, j, k);
        M_(C, j, i) = t / M_(L, i, i);
      }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < j; ++i) {
        double s = 0.5 * (M_(C, i, j) + M_(C, j, i));
        M_(C, i, j) = s;
        M_(C, j, i) = s;
      }
    for (int i = 0; i < n; ++i) M_(Q, i, i) = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
      double off = 0.0, tot = 0.0;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double v = M_(C, i, j) * M_(C, i, j);
          tot += v;
          if (i != j) off += v;
        }
      if (off <= 1e-34 * (tot > 0 ? tot : 1)) break;
      for (int p = 0; p < n - 1; ++p)
        for (int q = p + 1; q < n; ++q) {
          double apq = M_(C, p, q);
          if (apq == 0.0) continue;
          double app = M_(C, p, p), aqq = M_(C, q, q);
          double theta = (aqq - app) / (2.0 * apq);
          double t = (theta >= 0 ? 1.0 : -1.0) /
                     (fabs(theta) + sqrt(theta * theta + 1.0));
          double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
          for (int k = 0; k < n; ++k) {
            double ckp = M_(C, k, p), ckq = M_(C, k, q);
            M_(C, k, p) = cs * ckp - sn * ckq;
            M_(C, k, q) = sn * ckp + cs * ckq;
          }
          for (int k = 0; k < n; ++k) {
            double cpk = M_(C, p, k), cqk = M_(C, q, k);
            M_(C, p, k) = cs * cpk - sn * cqk;
            M_(C, q, k) = sn * cpk + cs * cqk;
          }
          for (int k = 0; k < n; ++k) {
            double qkp = M_(Q, k, p), qkq = M_(Q, k, q);
            M_(Q, k, p) = cs * qkp - sn * qkq;
            M_(Q, k, q) = sn * qkp + cs * qkq;
          }
        }
    }
    /* sort ascending */
    int *ord = malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j)
        if (M_(C, ord[j], ord[j]) < M_(C, ord[i], ord[i])) {
          int t = ord[i];
          ord[i] = ord[j];
          ord[j] = t;
        }
    /* X = L^-T Q (back substitution) */
    for (int jj = 0; jj < n; ++jj) {
      int j = ord[jj];
      lam[jj] = M_(C, j, j);
      for (int i = n - 1; i >= 0; --i) {
        double t = M_(Q, i, j);
        for (int k = i + 1; k < n; ++k) t -= M_(L, k, i) * M_(a, k, jj);
        M_(a, i, jj) = t / M_(L, i, i);
      }
    }
    free(ord);
  }
#undef M_
  free(L);
  free(C);
  free(Q);
  free(T);
  return info;
}

static void mg_free(orc_mg *m) {
  for (int l = 0; l < 8; ++l) {
    free(m->ah[l]); free(m->bh[l]); free(m->dh[l]); free(m->zh[l]);
    free(m->jh[l]); free(m->jht[l]);
    orc_gs_free(m->gsh[l]); orc_gs_free(m->gsh_schwarz[l]);
    free(m->rstr_wt[l]); free(m->fast_s[l]); free(m->fast_d[l]);
    free(m->schwarz_wt[l]); free(m->mask[l]);
  }
  free(m->work); free(m->work2); free(m->e); free(m->w); free(m->r);
  memset(m, 0, sizeof(*m));
}

static orc_gs *setupds(const orc_ctx *c, int nx) {
  long n = (long)nx * nx * nx * c->nelt;
  int64_t *glo = malloc(sizeof(int64_t) * n);
  orc_set_vert_box(glo, nx, c->nelt, c->nelx, c->nely, c->nelz, c->lglel);
  orc_gs *h = orc_gs_setup(glo, (int)n);
  free(glo);
  return h;
}

/* get_bcs, hsmg.f:605-642 */
static void get_bcs(const orc_ctx *c, int ie, int *lbr, int *rbr, int *lbs,
                    int *rbs, int *lbt, int *rbt) {
  int nelx = c->nelx, nely = c->nely, nelz = c->nelz, nelxy = nelx * nely;
  int ngl = c->lglel[ie - 1];
  int ir = 1 + (ngl - 1) / nelxy;
  int iq = mod1(ngl, nelxy);
  iq = 1 + (iq - 1) / nelx;
  int ip = mod1(ngl, nelx);
  *lbr = *rbr = *lbs = *rbs = *lbt = *rbt = 0;
  if (ip % nelx == 1 || nelx == 1) *lbr = 1;
  if (ip % nelx == 0) *rbr = 1;
  if (iq % nely == 1 || nely == 1) *lbs = 1;
  if (iq % nely == 0) *rbs = 1;
  if (ir % nelz == 1 || nelz == 1) *lbt = 1;
  if (ir % nelz == 0) *rbt = 1;
}

/* h1mg_setup_fast1d_a, hsmg.f:403-445; a is (0:n+2)^2 column-major */
static void fast1d_a(double *a, int lbc, int rbc, double ll, double lm,
                     double lr, const double *ah, int n) {
  int na = n + 3;
#define A_(i, j) a[(i) + (j) * na]
#define AH(i, j) ah[(i) + (j) * (n + 1)]
  int i0 = 0, i1 = n;
  if (lbc == 1) i0 = 1;
  if (rbc == 1) i1 = n - 1;
  for (int i = 0; i < na * na; ++i) a[i] = 0.;
  double fac = 2.0 / lm;
  A_(1, 1) = 1.0;
  A_(n + 1, n + 1) = 1.0;
  for (int j = i0; j <= i1; ++j)
    for (int i = i0; i <= i1; ++i) A_(i + 1, j + 1) = fac * AH(i, j);
  if (lbc == 0) {
    fac = 2.0 / ll;
    A_(0, 0) = fac * AH(n - 1, n - 1);
    A_(1, 0) = fac * AH(n, n - 1);
    A_(0, 1) = fac * AH(n - 1, n);
    A_(1, 1) = A_(1, 1) + fac * AH(n, n);
  } else {
    A_(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 2.0 / lr;
    A_(n + 1, n + 1) = A_(n + 1, n + 1) + fac * AH(0, 0);
    A_(n + 2, n + 1) = fac * AH(1, 0);
    A_(n + 1, n + 2) = fac * AH(0, 1);
    A_(n + 2, n + 2) = fac * AH(1, 1);
  } else {
    A_(n + 2, n + 2) = 1.0;
  }
#undef A_
#undef AH
}

/* h1mg_setup_fast1d_b, hsmg.f:447-481 */
static void fast1d_b(double *b, int lbc, int rbc, double ll, double lm,
                     double lr, const double *bh, int n) {
  int na = n + 3;
#define B_(i, j) b[(i) + (j) * na]
  int i0 = 0, i1 = n;
  if (lbc == 1) i0 = 1;
  if (rbc == 1) i1 = n - 1;
  for (int i = 0; i < na * na; ++i) b[i] = 0.;
  double fac = 0.5 * lm;
  B_(1, 1) = 1.0;
  B_(n + 1, n + 1) = 1.0;
  for (int i = i0; i <= i1; ++i) B_(i + 1, i + 1) = fac * bh[i];
  if (lbc == 0) {
    fac = 0.5 * ll;
    B_(0, 0) = fac * bh[n - 1];
    B_(1, 1) = B_(1, 1) + fac * bh[n];
  } else {
    B_(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 0.5 * lr;
    B_(n + 1, n + 1) = B_(n + 1, n + 1) + fac * bh[0];
    B_(n + 2, n + 2) = fac * bh[1];
  } else {
    B_(n + 2, n + 2) = 1.0;
  }
#undef B_
}

/* h1mg_setup_fast1d, hsmg.f:380-401; s is (nl,nl,2) */
static int fast1d(double *s, double *lam, int nl, int lbc, int rbc, double ll,
                  double lm, double lr, const double *ah, const double *bh,
                  int n) {
  double *b = malloc(sizeof(double) * nl * nl);
  fast1d_a(s, lbc, rbc, ll, lm, lr, ah, n);
  fast1d_b(b, lbc, rbc, ll, lm, lr, bh, n);
  int info = orc_generalev(s, b, lam, nl);
  free(b);
  /* row_zero, hsmg.f:525-532 */
#define ROWZ(e) for (int j = 0; j < nl; ++j) s[(e - 1) + j * nl] = 0.
  if (lbc > 0) ROWZ(1);
  if (lbc == 1) ROWZ(2);
  if (rbc > 0) ROWZ(nl);
  if (rbc == 1) ROWZ(nl - 1);
#undef ROWZ
  /* transpose(s(1,1,2), nl, s, nl), prox_setup.f:54-63 */
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) s[nl * nl + i + j * nl] = s[j + i * nl];
  return info;
}

static double vlmax(const double *v, int n) {
  double t = -99.0e20;
  for (int i = 0; i < n; ++i) t = t > v[i] ? t : v[i];
  return t;
}

/* h1mg_setup_fast, hsmg.f:285-378 */
static int setup_fast(orc_ctx *c, double *s, double *d, int nl,
                      const double *ah, const double *bh, int n) {
  int nx1 = c->nx1, nelt = c->nelt;
  long nxyz = (long)nx1 * nx1 * nx1;
  double *l = calloc((size_t)nxyz * nelt, sizeof(double));
  double lm = 2.0;
#define L_(i, j, k, e) l[((i) - 1) + (long)nx1 * ((j) - 1) + (long)nx1 * nx1 * ((k) - 1) + nxyz * (e)]
  for (int ie = 0; ie < nelt; ++ie) {
    L_(1, 2, 2, ie) = lm;
    L_(nx1, 2, 2, ie) = lm;
    L_(2, 1, 2, ie) = lm;
    L_(2, nx1, 2, ie) = lm;
    L_(2, 2, 1, ie) = lm;
    L_(2, 2, nx1, ie) = lm;
  }
  orc_dssum(c, l);
  int info = 0;
  double *lr = malloc(sizeof(double) * nl), *ls = malloc(sizeof(double) * nl),
         *lt = malloc(sizeof(double) * nl);
  for (int ie = 0; ie < nelt && !info; ++ie) {
    double llr = L_(1, 2, 2, ie) - lm, lrr = L_(nx1, 2, 2, ie) - lm;
    double lls = L_(2, 1, 2, ie) - lm, lrs = L_(2, nx1, 2, ie) - lm;
    double llt = L_(2, 2, 1, ie) - lm, lrt = L_(2, 2, nx1, ie) - lm;
    int lbr, rbr, lbs, rbs, lbt, rbt;
    get_bcs(c, ie + 1, &lbr, &rbr, &lbs, &rbs, &lbt, &rbt);
    double *se = s + (long)nl * nl * 2 * 3 * ie;
    info |= fast1d(se, lr, nl, lbr, rbr, llr, lm, lrr, ah, bh, n);
    info |= fast1d(se + 2 * nl * nl, ls, nl, lbs, rbs, lls, lm, lrs, ah, bh, n);
    info |= fast1d(se + 4 * nl * nl, lt, nl, lbt, rbt, llt, lm, lrt, ah, bh, n);
    double eps = 1.e-5 * (vlmax(lr + 1, nl - 2) + vlmax(ls + 1, nl - 2) +
                          vlmax(lt + 1, nl - 2));
    double *de = d + (long)nl * nl * nl * ie;
    int il = 0;
    for (int k = 0; k < nl; ++k)
      for (int j = 0; j < nl; ++j)
        for (int i = 0; i < nl; ++i) {
          double diag = lr[i] + ls[j] + lt[k];
          de[il++] = diag > eps ? 1.0 / diag : 0.0;
        }
  }
#undef L_
  free(lr); free(ls); free(lt); free(l);
  return info;
}

/* h1mg_setup_rstr_wt, hsmg.f:201-249 */
static void setup_rstr_wt(orc_ctx *c, double *wt, int nx, orc_gs *gsh) {
  int nelt = c->nelt, ny = nx, nz = nx;
  long nxyz = (long)nx * ny * nz;
  double *w = calloc((size_t)nxyz * nelt, sizeof(double));
#define W_(i, j, k, e) w[((i) - 1) + (long)nx * ((j) - 1) + (long)nx * ny * ((k) - 1) + nxyz * (e)]
#define WT(a, b, s, d, e) wt[((a) - 1) + (long)nx * ((b) - 1) + (long)nx * nz * ((s) - 1) + (long)nx * nz * 2 * ((d) - 1) + (long)nx * nz * 6 * (e)]
  for (int ie = 0; ie < nelt; ++ie) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) { W_(i, j, 1, ie) = 1.0; W_(i, j, nz, ie) = 1.0; }
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) { W_(i, 1, k, ie) = 1.0; W_(i, ny, k, ie) = 1.0; }
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) { W_(1, j, k, ie) = 1.0; W_(nx, j, k, ie) = 1.0; }
  }
  orc_gs_op(gsh, w, 1, 1, 0);
  for (int ie = 0; ie < nelt; ++ie) {
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        WT(j, k, 1, 1, ie) = 1.0 / W_(1, j, k, ie);
        WT(j, k, 2, 1, ie) = 1.0 / W_(nx, j, k, ie);
      }
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        WT(i, k, 1, 2, ie) = 1.0 / W_(i, 1, k, ie);
        WT(i, k, 2, 2, ie) = 1.0 / W_(i, ny, k, ie);
      }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        WT(i, j, 1, 3, ie) = 1.0 / W_(i, j, 1, ie);
        WT(i, j, 2, 3, ie) = 1.0 / W_(i, j, nz, ie);
      }
  }
#undef W_
#undef WT
  free(w);
}

/* h1mg_extrude, hsmg.f:1246-1283 */
static void extrude(const orc_ctx *c, double *arr1, int l1, double f1,
                    const double *arr2, int l2, double f2, int nx) {
  long nxyz = (long)nx * nx * nx;
  int i0 = 2, i1 = nx - 1;
#define X1(i, j, k) arr1[((i) - 1) + (long)nx * ((j) - 1) + (long)nx * nx * ((k) - 1) + off]
#define X2(i, j, k) arr2[((i) - 1) + (long)nx * ((j) - 1) + (long)nx * nx * ((k) - 1) + off]
  for (int ie = 0; ie < c->nelt; ++ie) {
    long off = nxyz * ie;
    for (int k = i0; k <= i1; ++k)
      for (int j = i0; j <= i1; ++j) {
        X1(l1 + 1, j, k) = FMAC(f2, X2(l2 + 1, j, k), f1 * X1(l1 + 1, j, k));
        X1(nx - l1, j, k) = FMAC(f2, X2(nx - l2, j, k), f1 * X1(nx - l1, j, k));
      }
    for (int k = i0; k <= i1; ++k)
      for (int i = i0; i <= i1; ++i) {
        X1(i, l1 + 1, k) = FMAC(f2, X2(i, l2 + 1, k), f1 * X1(i, l1 + 1, k));
        X1(i, nx - l1, k) = FMAC(f2, X2(i, nx - l2, k), f1 * X1(i, nx - l1, k));
      }
    for (int j = i0; j <= i1; ++j)
      for (int i = i0; i <= i1; ++i) {
        X1(i, j, l1 + 1) = FMAC(f2, X2(i, j, l2 + 1), f1 * X1(i, j, l1 + 1));
        X1(i, j, nx - l1) = FMAC(f2, X2(i, j, nx - l2), f1 * X1(i, j, nx - l1));
      }
  }
#undef X1
#undef X2
}

/* h1mg_schwarz_toext3d / toreg3d, hsmg.f:1207-1244 */
static void toext3d(const orc_ctx *c, double *a, const double *b, int n) {
  int m = n + 2;
  long m3 = (long)m * m * m, n3 = (long)n * n * n;
  memset(a, 0, sizeof(double) * m3 * c->nelt);
  for (int ie = 0; ie < c->nelt; ++ie)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
          a[(i + 1) + (long)m * (j + 1) + (long)m * m * (k + 1) + m3 * ie] =
              b[i + (long)n * j + (long)n * n * k + n3 * ie];
}
static void toreg3d(const orc_ctx *c, double *b, const double *a, int n) {
  int m = n + 2;
  long m3 = (long)m * m * m, n3 = (long)n * n * n;
  for (int ie = 0; ie < c->nelt; ++ie)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
          b[i + (long)n * j + (long)n * n * k + n3 * ie] =
              a[(i + 1) + (long)m * (j + 1) + (long)m * m * (k + 1) + m3 * ie];
}

/* h1mg_setup_schwarz_wt3d_1 / _2, hsmg.f:572-688 */
static void setup_schwarz_wt(orc_ctx *c, int l) {
  orc_mg *m = &c->mg;
  int nh = m->nh[l], en = nh + 2, nelt = c->nelt;
  long ns = (long)en * en * en * nelt;
  double *A = m->work, *B = m->work + ns;
  for (long i = 0; i < ns; ++i) B[i] = 1.0;
  extrude(c, A, 0, 0.0, B, 0, 1.0, en);
  orc_gs_op(m->gsh_schwarz[l], B, 1, 1, 0);
  extrude(c, B, 0, 1.0, A, 0, -1.0, en);
  extrude(c, B, 2, 1.0, B, 0, 1.0, en);
  toreg3d(c, A, B, nh);
  orc_gs_op(m->gsh[l], A, 1, 1, 0);
  int n = nh;
  long nxyz = (long)n * n * n;
  double *wt = m->schwarz_wt[l];
#define WK(i, j, k) work[((i) - 1) + (long)n * ((j) - 1) + (long)n * n * ((k) - 1)]
#define WT(a, b, s, d, e) wt[((a) - 1) + (long)n * ((b) - 1) + (long)n * n * ((s) - 1) + (long)n * n * 4 * ((d) - 1) + (long)n * n * 12 * (e)]
  for (int ie = 0; ie < nelt; ++ie) {
    const double *work = A + nxyz * ie;
    for (int k = 1; k <= n; ++k)
      for (int j = 1; j <= n; ++j) {
        WT(j, k, 1, 1, ie) = 1.0 / WK(1, j, k);
        WT(j, k, 2, 1, ie) = 1.0 / WK(2, j, k);
        WT(j, k, 3, 1, ie) = 1.0 / WK(n - 1, j, k);
        WT(j, k, 4, 1, ie) = 1.0 / WK(n, j, k);
      }
    for (int k = 1; k <= n; ++k)
      for (int i = 1; i <= n; ++i) {
        WT(i, k, 1, 2, ie) = 1.0 / WK(i, 1, k);
        WT(i, k, 2, 2, ie) = 1.0 / WK(i, 2, k);
        WT(i, k, 3, 2, ie) = 1.0 / WK(i, n - 1, k);
        WT(i, k, 4, 2, ie) = 1.0 / WK(i, n, k);
      }
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) {
        WT(i, j, 1, 3, ie) = 1.0 / WK(i, j, 1);
        WT(i, j, 2, 3, ie) = 1.0 / WK(i, j, 2);
        WT(i, j, 3, 3, ie) = 1.0 / WK(i, j, n - 1);
        WT(i, j, 4, 3, ie) = 1.0 / WK(i, j, n);
      }
  }
#undef WK
#undef WT
}

/* h1mg_setup_mask, hsmg.f:853-911 (maskit's build branch per element) */
static int *setup_mask(orc_ctx *c, int nx) {
  int nel = c->nelt;
  long nxyz = (long)nx * nx * nx, n = nxyz * nel;
  double *w = malloc(sizeof(double) * n);
  for (long i = 0; i < n; ++i) w[i] = 1.0;
  double *cm = calloc((size_t)n + 2, sizeof(double));
  maskit_ref(c, w, cm, nx);
  free(cm);
  int *mask = malloc(sizeof(int) * (n + 2 * nel + 2));
  /* mask is 1-based in the reference: mask(e) = nel+nm ... */
#define MK(i) mask[(i) - 1]
  int nm = 1;
  for (int e = 1; e <= nel; ++e) {
    MK(e) = nel + nm;
    int count = 0, ptr = MK(e);
    for (long i = 1; i <= nxyz; ++i)
      if (w[(i - 1) + nxyz * (e - 1)] == 0) {
        nm = nm + 1;
        count = count + 1;
        ptr = ptr + 1;
        MK(ptr) = (int)(i + nxyz * (e - 1));
      }
    ptr = MK(e);
    MK(ptr) = count;
    nm = nm + 1;
  }
#undef MK
  free(w);
  return mask;
}

/* h1mg_mask / mg_mask_e, hsmg.f:1180-1205 */
static void mg_mask(const orc_ctx *c, double *w, const int *mask) {
  for (int e = 1; e <= c->nelt; ++e) {
    int im = mask[e - 1];
    const int *mk = mask + (im - 1);
    int n = mk[0];
    for (int i = 1; i <= n; ++i) w[mk[i] - 1] = 0.;
  }
}

/* h1mg_setup_intpm, hsmg.f:138-152: jh (nf x nc) */
static void setup_intpm(double *jh, const double *zf, const double *zc, int nf,
                        int nc) {
  double w[2 * NMAX + 2];
  for (int i = 0; i < nf; ++i) {
    orc_fd_weights_full(zf[i], zc, nc - 1, 1, w);
    for (int j = 0; j < nc; ++j) jh[i + j * nf] = w[j];
  }
}

/* h1mg_setup, hsmg.f:3-29; level choice h1mg_setup_mg_nx hsmg.f:45-97 */
int orc_h1mg_setup(orc_ctx *c, const int *orders, int nlev) {
  orc_mg *m = &c->mg;
  mg_free(m);
  int nx1 = c->nx1;
  if (!orders) {
    static const int mgn2[10] = {1, 2, 2, 2, 2, 3, 3, 5, 5, 5};
    int lmax = 3;
    if (nx1 == 4) lmax = 2;
    if (nx1 > 10) return -1; /* hsmg.f:65 reads the undefined lx2 here */
    int mgnx2 = mgn2[nx1 - 1];
    if (nx1 == 8) mgnx2 = 3;
    mgnx2 = mgnx2 < 3 ? mgnx2 : 3;
    m->nx[1] = 1;
    m->nx[2] = mgnx2;
    m->nx[3] = mgnx2 + 1;
    m->nx[lmax] = nx1 - 1;
    m->nlev = lmax;
  } else {
    if (nlev < 2 || nlev > 7) return -1;
    for (int l = 1; l <= nlev; ++l) m->nx[l] = orders[l - 1];
    if (m->nx[nlev] != nx1 - 1) return -1;
    m->nlev = nlev;
  }
  int L = m->nlev, nelt = c->nelt;
  for (int l = 1; l <= L; ++l) {
    int n = m->nx[l], nh = n + 1;
    m->nh[l] = nh;
    m->ah[l] = malloc(sizeof(double) * nh * nh);
    m->bh[l] = malloc(sizeof(double) * nh);
    m->dh[l] = malloc(sizeof(double) * nh * nh);
    m->zh[l] = malloc(sizeof(double) * nh);
    double *cc = malloc(sizeof(double) * nh * nh);
    orc_semhat(m->ah[l], m->bh[l], cc, m->dh[l], m->zh[l], n);
    free(cc);
    m->ntot[l] = nh * nh * nh * nelt;
  }
  for (int l = 1; l < L; ++l) {
    int nf = m->nh[l + 1], nc = m->nh[l];
    m->jh[l] = malloc(sizeof(double) * nf * nc);
    m->jht[l] = malloc(sizeof(double) * nf * nc);
    setup_intpm(m->jh[l], m->zh[l + 1], m->zh[l], nf, nc);
    for (int j = 0; j < nc; ++j)
      for (int i = 0; i < nf; ++i) m->jht[l][j + i * nc] = m->jh[l][i + j * nf];
  }
  int maxext = 0;
  for (int l = 1; l <= L; ++l) {
    m->gsh[l] = setupds(c, m->nh[l]);
    m->gsh_schwarz[l] = setupds(c, m->nh[l] + 2);
    int e3 = (m->nh[l] + 2) * (m->nh[l] + 2) * (m->nh[l] + 2);
    if (e3 > maxext) maxext = e3;
  }
  m->work = calloc((size_t)2 * maxext * nelt, sizeof(double));
  m->work2 = calloc((size_t)2 * maxext * nelt, sizeof(double));
  for (int l = 1; l <= L; ++l) {
    int nh = m->nh[l];
    m->rstr_wt[l] = malloc(sizeof(double) * nh * nh * 2 * 3 * nelt);
    setup_rstr_wt(c, m->rstr_wt[l], nh, m->gsh[l]);
  }
  int info = 0;
  for (int l = 2; l <= L; ++l) {
    int nl = m->nh[l] + 2;
    m->fast_s[l] = malloc(sizeof(double) * nl * nl * 2 * 3 * nelt);
    m->fast_d[l] = malloc(sizeof(double) * nl * nl * nl * nelt);
    info |= setup_fast(c, m->fast_s[l], m->fast_d[l], nl, m->ah[l], m->bh[l],
                       m->nx[l]);
  }
  for (int l = 2; l <= L; ++l) {
    int nh = m->nh[l];
    m->schwarz_wt[l] = malloc(sizeof(double) * nh * nh * 4 * 3 * nelt);
    setup_schwarz_wt(c, l);
  }
  for (int l = L; l >= 1; --l) m->mask[l] = setup_mask(c, m->nh[l]);
  m->e = calloc((size_t)2 * c->n, sizeof(double));
  m->w = calloc((size_t)c->n, sizeof(double));
  m->r = calloc((size_t)c->n, sizeof(double));
  m->ready = 1;
  return info;
}

int orc_h1mg_nlev(const orc_ctx *c) { return c->mg.nlev; }
int orc_h1mg_order(const orc_ctx *c, int l) { return c->mg.nx[l]; }
void orc_h1mg_fdm_copy(const orc_ctx *c, int l, double *s, double *d) {
  int nl = c->mg.nh[l] + 2;
  memcpy(s, c->mg.fast_s[l], sizeof(double) * nl * nl * 6 * c->nelt);
  memcpy(d, c->mg.fast_d[l], sizeof(double) * nl * nl * nl * c->nelt);
}

/* tensor apply v = [C (x) B (x) A] u for one element, hsmg.f:1320-1338 */
static void tnsr3d_el(double *v, int nv, const double *u, int nu,
                      const double *A, const double *Bt, const double *Ct,
                      double *work, double *work2) {
  orc_mxm(A, nv, u, nu, work, nu * nu);
  for (int i = 0; i < nu; ++i)
    orc_mxm(work + (long)nv * nu * i, nv, Bt, nu, work2 + (long)nv * nv * i, nv);
  orc_mxm(work2, nv * nv, Ct, nu, v, nv);
}

/* h1mg_do_fast, hsmg.f:1297-1318 (clobbers r) */
static void do_fast(const orc_ctx *c, double *e, double *r, const double *s,
                    const double *d, int nl) {
  long nn = (long)nl * nl * nl, ss = (long)nl * nl;
  double *work = malloc(sizeof(double) * nn), *work2 = malloc(sizeof(double) * nn);
  for (int ie = 0; ie < c->nelt; ++ie) {
    const double *se = s + ss * 6 * ie;
    double *ee = e + nn * ie, *re = r + nn * ie;
    /* s(1,2,1)=S_r^T, s(1,1,2)=S_s, s(1,1,3)=S_t */
    tnsr3d_el(ee, nl, re, nl, se + ss, se + 2 * ss, se + 4 * ss, work, work2);
    for (long i = 0; i < nn; ++i) re[i] = d[nn * ie + i] * ee[i];
    /* s(1,1,1)=S_r, s(1,2,2)=S_s^T, s(1,2,3)=S_t^T */
    tnsr3d_el(ee, nl, re, nl, se, se + 3 * ss, se + 5 * ss, work, work2);
  }
  free(work);
  free(work2);
}

/* h1mg_schwarz_wt3d2, hsmg.f:1144-1178 (multiplies by sqrt(wt)) */
static void schwarz_wt3d2(const orc_ctx *c, double *e, const double *wt, int n) {
  long nxyz = (long)n * n * n;
#define E_(i, j, k) ee[((i) - 1) + (long)n * ((j) - 1) + (long)n * n * ((k) - 1)]
#define WT(a, b, s, d) we[((a) - 1) + (long)n * ((b) - 1) + (long)n * n * ((s) - 1) + (long)n * n * 4 * ((d) - 1)]
  for (int ie = 0; ie < c->nelt; ++ie) {
    double *ee = e + nxyz * ie;
    const double *we = wt + (long)n * n * 12 * ie;
    for (int k = 1; k <= n; ++k)
      for (int j = 1; j <= n; ++j) {
        E_(1, j, k) = E_(1, j, k) * sqrt(WT(j, k, 1, 1));
        E_(2, j, k) = E_(2, j, k) * sqrt(WT(j, k, 2, 1));
        E_(n - 1, j, k) = E_(n - 1, j, k) * sqrt(WT(j, k, 3, 1));
        E_(n, j, k) = E_(n, j, k) * sqrt(WT(j, k, 4, 1));
      }
    for (int k = 1; k <= n; ++k)
      for (int i = 3; i <= n - 2; ++i) {
        E_(i, 1, k) = E_(i, 1, k) * sqrt(WT(i, k, 1, 2));
        E_(i, 2, k) = E_(i, 2, k) * sqrt(WT(i, k, 2, 2));
        E_(i, n - 1, k) = E_(i, n - 1, k) * sqrt(WT(i, k, 3, 2));
        E_(i, n, k) = E_(i, n, k) * sqrt(WT(i, k, 4, 2));
      }
    for (int j = 3; j <= n - 2; ++j)
      for (int i = 3; i <= n - 2; ++i) {
        E_(i, j, 1) = E_(i, j, 1) * sqrt(WT(i, j, 1, 3));
        E_(i, j, 2) = E_(i, j, 2) * sqrt(WT(i, j, 2, 3));
        E_(i, j, n - 1) = E_(i, j, n - 1) * sqrt(WT(i, j, 3, 3));
        E_(i, j, n) = E_(i, j, n) * sqrt(WT(i, j, 4, 3));
      }
  }
#undef E_
#undef WT
}

/* h1mg_schwarz_part1, hsmg.f:1053-1095 */
static void schwarz_part1(orc_ctx *c, double *e, double *r, int l) {
  orc_mg *m = &c->mg;
  int nh = m->nh[l], en = nh + 2;
  long ns = (long)en * en * en * c->nelt;
  double *A = m->work, *B = m->work + ns;
  mg_mask(c, r, m->mask[l]);
  toext3d(c, A, r, nh);
  extrude(c, A, 0, 0.0, A, 2, 1.0, en);
  orc_gs_op(m->gsh_schwarz[l], A, 1, 1, 0);
  extrude(c, A, 0, 1.0, A, 2, -1.0, en);
  do_fast(c, B, A, m->fast_s[l], m->fast_d[l], en);
  extrude(c, A, 0, 0.0, B, 0, 1.0, en);
  orc_gs_op(m->gsh_schwarz[l], B, 1, 1, 0);
  extrude(c, B, 0, 1.0, A, 0, -1.0, en);
  extrude(c, B, 2, 1.0, B, 0, 1.0, en);
  toreg3d(c, e, B, nh);
  orc_gs_op(m->gsh[l], e, 1, 1, 0);
  mg_mask(c, e, m->mask[l]);
}

/* h1mg_schwarz, hsmg.f:1036-1051.  Its first h1mg_schwarz_wt call scales the
 * output array before part1 overwrites every entry of it, so it has no effect
 * on the result and is not repeated here. */
static void mg_schwarz(orc_ctx *c, double *e, double *r, double sigma, int l) {
  orc_mg *m = &c->mg;
  schwarz_part1(c, e, r, l);
  schwarz_wt3d2(c, e, m->schwarz_wt[l], m->nh[l]);
  for (int i = 0; i < m->ntot[l]; ++i) e[i] = e[i] * sigma;
}

/* h1mg_do_wt, hsmg.f:1362-1391 */
static void do_wt(const orc_ctx *c, double *u, const double *wt, int nx) {
  int ny = nx, nz = nx;
  long nxyz = (long)nx * ny * nz;
#define U_(i, j, k) ue[((i) - 1) + (long)nx * ((j) - 1) + (long)nx * ny * ((k) - 1)]
#define WT(a, b, s, d) we[((a) - 1) + (long)nx * ((b) - 1) + (long)nx * nz * ((s) - 1) + (long)nx * nz * 2 * ((d) - 1)]
  for (int ie = 0; ie < c->nelt; ++ie) {
    double *ue = u + nxyz * ie;
    const double *we = wt + (long)nx * nz * 6 * ie;
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        U_(1, j, k) = U_(1, j, k) * WT(j, k, 1, 1);
        U_(nx, j, k) = U_(nx, j, k) * WT(j, k, 2, 1);
      }
    for (int k = 1; k <= nz; ++k)
      for (int i = 2; i <= nx - 1; ++i) {
        U_(i, 1, k) = U_(i, 1, k) * WT(i, k, 1, 2);
        U_(i, ny, k) = U_(i, ny, k) * WT(i, k, 2, 2);
      }
    for (int j = 2; j <= ny - 1; ++j)
      for (int i = 2; i <= nx - 1; ++i) {
        U_(i, j, 1) = U_(i, j, 1) * WT(i, j, 1, 3);
        U_(i, j, nz) = U_(i, j, nz) * WT(i, j, 2, 3);
      }
  }
#undef U_
#undef WT
}

/* h1mg_tnsr1_3d, hsmg.f:1402-1434: in-place v = [Ct (x) Bt (x) A] u, element
 * order reversed when the output grows */
static void tnsr1_3d(const orc_ctx *c, double *v, int nv, int nu,
                     const double *A, const double *Bt, const double *Ct) {
  int nelt = c->nelt;
  int e0 = 1, es = 1, ee = nelt;
  if (nv > nu) { e0 = nelt; es = -1; ee = 1; }
  long nu3 = (long)nu * nu * nu, nv3 = (long)nv * nv * nv;
  long big = (nu3 > nv3 ? nu3 : nv3) * 2;
  double *work = malloc(sizeof(double) * big), *work2 = malloc(sizeof(double) * big);
  for (int e = e0;; e += es) {
    long iu = (e - 1) * nu3, iv = (e - 1) * nv3;
    orc_mxm(A, nv, v + iu, nu, work, nu * nu);
    for (int i = 0; i < nu; ++i)
      orc_mxm(work + (long)nv * nu * i, nv, Bt, nu, work2 + (long)nv * nv * i, nv);
    orc_mxm(work2, nv * nv, Ct, nu, v + iv, nv);
    if (e == ee) break;
  }
  free(work);
  free(work2);
}

/* h1mg_rstr, hsmg.f:1340-1360 (l is the coarse level) */
static void mg_rstr(orc_ctx *c, double *r, int l, int ifdssum) {
  orc_mg *m = &c->mg;
  do_wt(c, r, m->rstr_wt[l + 1], m->nh[l + 1]);
  tnsr1_3d(c, r, m->nh[l], m->nh[l + 1], m->jht[l], m->jh[l], m->jh[l]);
  if (ifdssum) orc_gs_op(m->gsh[l], r, 1, 1, 0);
}

/* h1mg_intp + h1mg_tnsr3d, hsmg.f:1436-1475 (l is the coarse level) */
static void mg_intp(orc_ctx *c, double *uf, const double *uc, int l) {
  orc_mg *m = &c->mg;
  int nv = m->nh[l + 1], nu = m->nh[l];
  long nu3 = (long)nu * nu * nu, nv3 = (long)nv * nv * nv;
  long big = (nu3 > nv3 ? nu3 : nv3) * 2;
  double *work = malloc(sizeof(double) * big), *work2 = malloc(sizeof(double) * big);
  for (int ie = 0; ie < c->nelt; ++ie)
    tnsr3d_el(uf + nv3 * ie, nv, uc + nu3 * ie, nu, m->jh[l], m->jht[l],
              m->jht[l], work, work2);
  free(work);
  free(work2);
}

/* h1mg_solve, hsmg.f:960-1034.  Note: the Schwarz step masks rhs in place. */
void orc_h1mg_solve(orc_ctx *c, double *z, double *rhs, int nn) {
  (void)nn;
  orc_mg *m = &c->mg;
  double sigma = 1.;
  int l = m->nlev;
  int n = m->ntot[l];
  long is = 0; /* 0-based offset into e */
  double *e = m->e, *w = m->w, *r = m->r;
  mg_schwarz(c, z, rhs, sigma, l);
  memcpy(r, rhs, sizeof(double) * n);
  for (l = m->nlev - 1; l >= 2; --l) {
    is = is + n;
    n = m->ntot[l];
    mg_rstr(c, r, l, 1);
    mg_schwarz(c, e + is, r, sigma, l);
  }
  is = is + n;
  mg_rstr(c, r, 1, 0);
  mg_mask(c, r, m->mask[1]);
  /* hsmg_coarse_solve, hsmg.f:945-957 */
  memcpy(e + is, r, sizeof(double) * m->ntot[1]);
  orc_gs_op(m->gsh[1], e + is, 1, 1, 0);
  mg_mask(c, e + is, m->mask[1]);
  for (l = 2; l <= m->nlev - 1; ++l) {
    long im = is;
    is = is - n;
    n = m->ntot[l];
    mg_intp(c, w, e + im, l - 1);
    for (int i = 0; i < n; ++i) e[is + i] = e[is + i] + w[i];
  }
  l = m->nlev;
  n = m->ntot[l];
  long im = is;
  mg_intp(c, w, e + im, l - 1);
  for (int i = 0; i < n; ++i) z[i] = z[i] + w[i];
}

// nb_abi.cpp -- the C ABI of the library (include/nekbone_gb300.h).
//
// The drop-in entry points keep the reference's Fortran signatures: host
// arrays in, host arrays out, the work done by CUDA kernels in between.  The
// values the Fortran routines read from common blocks (/dimn/, /hcglb/,
// /dxyz/, /comm_handles/, /mymask/, /cflops/) live in one library-wide state
// published through nekbone_common_ -- like the reference, the library is
// single-threaded and not re-entrant (jl's handle table and static buffer
// are global too, jl/gs.c:36,1156-1158).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <algorithm>
#include <thread>
#include <vector>

#include "../../include/nekbone_gb300.h"
#include "nb_mg.h"
#include "nb_solver.h"

namespace nb {

int dev_mxm(const double *a, int n1, const double *b, int n2, double *c,
            int n3, cudaStream_t s);
int dev_local_grad3(double *ur, double *us, double *ut, const double *u,
                    int n, const double *D, const double *Dt, cudaStream_t s);
int dev_local_grad3_t(double *u, const double *ur, const double *us,
                      const double *ut, int n, const double *D,
                      const double *Dt, double *w, cudaStream_t s);
int dev_setup_g(const Operator &op, double *g, cudaStream_t s);
int dev_rhs_uniform(const Operator &op, double *f, const double *c,
                    uint64_t seed, cudaStream_t s);
int dev_setup_g_deformed(const Operator &op, double *g, uint64_t seed, double amp,
                         cudaStream_t s);
int dev_residual(const Operator &op, double *r, const double *f,
                 const double *w, long n, cudaStream_t s);
int dev_axpy_f32(double *x, const float *e, double scale, long n, cudaStream_t s);
int dev_scale_to_f32(float *y, const double *r, double scale, long n, cudaStream_t s);

// ---------------------------------------------------------------- errors --
namespace {
int g_status = 0;
int g_mode = 0;
char g_msg[1024] = {0};
}  // namespace

int fail(int status, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  g_status = status;
  if (g_mode == 0) {
    fprintf(stderr, "ERROR (nekbone_gb300): %s\n", g_msg);
    fflush(stderr);
    exit(1);
  }
  return status;
}
int last_status() { return g_status; }
const char *last_message() { return g_msg; }
void clear_status() {
  g_status = 0;
  g_msg[0] = 0;
}
int error_mode() { return g_mode; }
void set_error_mode(int m) { g_mode = m; }

// ----------------------------------------------------------- global state --
struct GsEntry {
  GsHost host;           // jl's maps; empty for a recognised box until needed
  GsDevice dev;
  int n = 0;
  // set_vert_box's numbering of a brick box, recognised by gs_setup_: the
  // maps were built on the device without a sort
  bool box = false;
  int lx = 0, nelx = 0, nely = 0, nelz = 0;
  int ensure_host() {
    if (!box || !host.map[0].empty()) return NB_OK;
    const long nelt = long(nelx) * nely * nelz;
    std::vector<int> lglel(nelt);
    for (long e = 0; e < nelt; ++e) lglel[e] = int(e + 1);
    std::vector<int64_t> glo(n);
    set_vert_box(glo.data(), lx, int(nelt), nelx, nely, lglel.data());
    gs_topology(glo.data(), n, &host);
    return NB_OK;
  }
};

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  int get(size_t bytes, void **out) {
    if (bytes > cap) {
      if (p) cudaFree(p);
      p = nullptr;
      cap = 0;
      NB_CUDA(cudaMalloc(&p, bytes));
      cap = bytes;
    }
    *out = p;
    return NB_OK;
  }
};

struct State {
  cudaStream_t s = nullptr;
  std::vector<std::unique_ptr<GsEntry>> gs;
  bool common_set = false;
  int nelx = 0, nely = 0, nelz = 0, nelt = 0, nx1 = 0, gsh = -1;
  std::vector<int> lglel;
  std::vector<double> dxm1;
  int mask_mode = 0;
  int order = 2;  // contraction form of the FP64 operator (2 fixed point)
  bool mgrid = false;
  double flop_a = 0.0, flop_cg = 0.0;
  std::unique_ptr<Operator> op;
  std::unique_ptr<Multigrid> mg;
  CgWork wk;
  DevBuf buf[12];
  int init() {
    if (!s) NB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamDefault));  // orders with the legacy default stream
    return NB_OK;
  }
};

State &st() {
  static State *S = new State();
  return *S;
}

template <typename T>
int dbuf(int slot, size_t count, T **out) {
  void *p = nullptr;
  NB_TRY(st().buf[slot].get(count * sizeof(T), &p));
  *out = static_cast<T *>(p);
  return NB_OK;
}

int check_common() {
  if (!st().common_set)
    return fail(NB_ERR_STATE, "mesh not published (call nekbone_common_ first)");
  return NB_OK;
}

GsEntry *gs_entry(int h, const char *func) {
  State &S = st();
  if (h < 0 || h >= int(S.gs.size()) || !S.gs[h]) {
    fail(NB_ERR_HANDLE, "%s: invalid handle", func);
    return nullptr;
  }
  return S.gs[h].get();
}

// Operator of the published mesh, built on first use.
int common_op(Operator **out) {
  State &S = st();
  NB_TRY(check_common());
  NB_TRY(S.init());
  if (!S.op) {
    GsEntry *g = gs_entry(S.gsh, "dssum");
    if (!g) return last_status();
    const long n = long(S.nelt) * S.nx1 * S.nx1 * S.nx1;
    if (g->n != n)
      return fail(NB_ERR_ARG, "gsh has %d points, the mesh has %ld", g->n, n);
    std::unique_ptr<Operator> op(new Operator());
    bool brick = g->box && g->lx == S.nx1 && g->nelx == S.nelx && g->nely == S.nely &&
                 g->nelz == S.nelz && setup_on_device();
    for (int e = 0; brick && e < S.nelt; ++e) brick = S.lglel[e] == e + 1;
    if (brick) {  // the box's topology on the device, as nb_mesh_create builds it
      NB_TRY(operator_base(op.get(), S.nelx, S.nely, S.nelz, S.nelt, S.nx1, S.lglel.data(),
                           S.dxm1.data(), S.mask_mode, S.s));
      NB_TRY(box_topology_device(op.get(), S.s));
    } else {
      NB_TRY(g->ensure_host());
      NB_TRY(operator_from(op.get(), S.nelx, S.nely, S.nelz, S.nelt, S.nx1,
                           S.lglel.data(), S.dxm1.data(), g->host, S.mask_mode, S.s));
    }
    op->order = S.order;
    S.op = std::move(op);
  }
  *out = S.op.get();
  return NB_OK;
}

int32_t wrap_mul(int32_t a, int32_t b) { return int32_t(uint32_t(a) * uint32_t(b)); }
int32_t wrap_add(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }

// flop_a increment of one ax call, in default-integer arithmetic (cg.f:122)
double ax_flops(int nx1, int nelt) {
  const int32_t nxyz = wrap_mul(wrap_mul(nx1, nx1), nx1);
  return double(wrap_mul(wrap_add(wrap_mul(19, nxyz), wrap_mul(wrap_mul(12, nx1), nxyz)), nelt));
}

int h2d(void *d, const void *h, size_t bytes) {
  NB_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st().s));
  return NB_OK;
}
int d2h(void *h, const void *d, size_t bytes) {
  NB_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st().s));
  return NB_OK;
}
int sync() {
  NB_CUDA(cudaStreamSynchronize(st().s));
  return NB_OK;
}

// ---------------------------------------------------- mgrid preconditioner --
struct MgPrecond : Precond {
  Multigrid *mg;
  explicit MgPrecond(Multigrid *m) : mg(m) {}
  int apply(double *z, double *r, cudaStream_t s) override {
    return mg_solve(*mg, z, r, s);
  }
  // FP32 smoother on a fully masked CG (mask mode 1: r is already zero
  // wherever the finest level masks, so the in-place mask of r is a no-op)
  float *r32_in() override {
    return mg->precision == 32 && mg->op->mask_mode == 1 ? mg->lv[mg->nlev].r_f : nullptr;
  }
  int apply_f32(cudaStream_t s) override { return mg_solve_f32(*mg, s); }
  const float *z32_out() override { return mg->z_f; }
};

cudaStream_t lib_stream() {
  st().init();
  return st().s;
}

}  // namespace nb

using namespace nb;

struct nb_mesh {
  Operator op;
  CgWork wk;
  std::unique_ptr<Multigrid> mg;
};

extern "C" {

int nekbone_last_status(void) { return last_status(); }
const char *nekbone_last_message(void) { return last_message(); }
void nekbone_clear_status(void) { clear_status(); }
void nekbone_set_error_mode(int mode) { set_error_mode(mode); }
int nekbone_version(void) { return 1; }

// ------------------------------------------------------------ common --
void nekbone_common_(const int *nelx, const int *nely, const int *nelz,
                     const int *nelt, const int *nx1, const int *lglel,
                     const double *dxm1, const int *gsh) {
  clear_status();
  State &S = st();
  if (*nelt <= 0 || *nx1 < 2) {
    fail(NB_ERR_ARG, "nekbone_common_: nelt=%d nx1=%d", *nelt, *nx1);
    return;
  }
  S.nelx = *nelx;
  S.nely = *nely;
  S.nelz = *nelz;
  S.nelt = *nelt;
  S.nx1 = *nx1;
  S.lglel.assign(lglel, lglel + *nelt);
  S.dxm1.assign(dxm1, dxm1 + (*nx1) * (*nx1));
  S.gsh = *gsh;
  S.common_set = true;
  S.op.reset();
  S.mg.reset();
}

void nekbone_mask_reset_(void) {
  State &S = st();
  if (S.op) {
    S.op->mask_built = S.op->mask_mode == 1;
    if (S.op->mask_mode == 0) operator_set_mask(S.op.get(), std::vector<int>());
  }
}

void nekbone_set_mask_mode_(const int *mode) {
  clear_status();
  if (*mode != 0 && *mode != 1) {
    fail(NB_ERR_ARG, "mask mode %d not 0 or 1", *mode);
    return;
  }
  st().mask_mode = *mode;
  st().op.reset();
  st().mg.reset();
}

void nekbone_set_mgrid_(const int *ifmgrid) { st().mgrid = *ifmgrid != 0; }

void nekbone_set_contraction_order_(const int *order) {
  clear_status();
  if (*order < 0 || *order > 2) {
    fail(NB_ERR_ARG, "contraction order %d not 0, 1 or 2", *order);
    return;
  }
  st().order = *order;
  if (st().op) st().op->order = *order;
}

void nekbone_get_flops_(double *flop_a, double *flop_cg) {
  *flop_a = st().flop_a;
  *flop_cg = st().flop_cg;
}
void nekbone_set_flops_(const double *flop_a, const double *flop_cg) {
  st().flop_a = *flop_a;
  st().flop_cg = *flop_cg;
}

// -------------------------------------------------------------- jl gs --
void gs_setup_(int *handle, const int64_t *glo_num, const int *n,
               const int *comm, const int *np) {
  (void)comm;
  clear_status();
  State &S = st();
  if (S.init()) return;
  if (*n < 0) {
    fail(NB_ERR_ARG, "gs_setup: n=%d", *n);
    return;
  }
  if (np && *np != 1) {
    fail(NB_ERR_UNSUPPORTED, "gs_setup: np=%d; one process per GPU is supported", *np);
    return;
  }
  std::unique_ptr<GsEntry> e(new GsEntry());
  e->n = *n;
  bool box = false;
  if (setup_on_device() &&
      box_numbering(glo_num, *n, &box, &e->lx, &e->nelx, &e->nely, &e->nelz, S.s))
    return;
  if (box) {  // no sort: the closed-form copies of each box point
    e->box = true;
    if (box_gs_device(e->lx, e->nelx, e->nely, e->nelz, &e->dev, S.s)) return;
  } else {
    gs_topology(glo_num, *n, &e->host);
    if (gs_upload(e->host, *n, &e->dev, S.s)) return;
  }
  S.gs.push_back(std::move(e));
  *handle = int(S.gs.size()) - 1;
}

void gs_op_(const int *handle, void *u, const int *dom, const int *op,
            const int *transpose) {
  clear_status();
  State &S = st();
  if (*dom < 1 || *dom > 4) {
    fail(NB_ERR_ARG, "gs_op: datatype %d not in valid range 1-4", *dom);
    return;
  }
  if (*op < 1 || *op > 4) {
    fail(NB_ERR_ARG, "gs_op: op %d not in valid range 1-4", *op);
    return;
  }
  GsEntry *g = gs_entry(*handle, "gs_op");
  if (!g) return;
  static const size_t sz[5] = {0, 8, 4, 4, 8};
  const size_t bytes = sz[*dom] * size_t(g->n);
  if (!bytes) return;
  void *d = nullptr;
  if (S.buf[0].get(bytes, &d)) return;
  if (h2d(d, u, bytes)) return;
  if (gs_exec(g->dev, d, *dom, *op, *transpose, S.s)) return;
  if (d2h(u, d, bytes)) return;
  sync();
}

void gs_free_(const int *handle) {
  clear_status();
  GsEntry *g = gs_entry(*handle, "gs_free");
  if (!g) return;
  gs_release(&g->dev);
  st().gs[*handle].reset();
}

void dssum_(double *f) {
  clear_status();
  if (check_common()) return;
  const int dom = 1, op = 1, tr = 0;
  gs_op_(&st().gsh, f, &dom, &op, &tr);
}

// ------------------------------------------------------------ math.f --
double glsc3_(const double *a, const double *b, const double *mult,
              const int *n) {
  clear_status();
  State &S = st();
  if (S.init()) return 0.0;
  const long nn = *n;
  if (nn <= 0) return 0.0;
  double *da, *db, *dm;
  if (dbuf(0, nn, &da) || dbuf(1, nn, &db) || dbuf(2, nn, &dm)) return 0.0;
  if (h2d(da, a, nn * 8) || h2d(db, b, nn * 8) || h2d(dm, mult, nn * 8)) return 0.0;
  CgWork &wk = S.wk;
  Operator dummy;
  dummy.n = nn;
  dummy.nelt = 1;
  if (wk.ensure(dummy, 1)) return 0.0;
  if (vec_glsc3<double>(da, db, dm, nn, wk, wk.dot_out, nullptr, 0, 0, S.s)) return 0.0;
  double v = 0.0;
  if (d2h(&v, wk.dot_out, 8) || sync()) return 0.0;
  return v;
}

void add2s1_(double *a, const double *b, const double *c1, const int *n) {
  clear_status();
  State &S = st();
  if (S.init() || *n <= 0) return;
  double *da, *db;
  if (dbuf(0, *n, &da) || dbuf(1, *n, &db)) return;
  if (h2d(da, a, *n * 8L) || h2d(db, b, *n * 8L)) return;
  if (vec_add2s1<double>(da, db, nullptr, *c1, *n, S.s)) return;
  if (d2h(a, da, *n * 8L)) return;
  sync();
}

void add2s2_(double *a, const double *b, const double *c1, const int *n) {
  clear_status();
  State &S = st();
  if (S.init() || *n <= 0) return;
  double *da, *db;
  if (dbuf(0, *n, &da) || dbuf(1, *n, &db)) return;
  if (h2d(da, a, *n * 8L) || h2d(db, b, *n * 8L)) return;
  if (vec_add2s2<double>(da, db, *c1, *n, S.s)) return;
  if (d2h(a, da, *n * 8L)) return;
  sync();
}

void mxm_(const double *a, const int *n1, const double *b, const int *n2,
          double *c, const int *n3) {
  clear_status();
  State &S = st();
  if (S.init()) return;
  if (*n1 <= 0 || *n2 <= 0 || *n3 <= 0) return;
  const long na = long(*n1) * *n2, nb_ = long(*n2) * *n3, nc = long(*n1) * *n3;
  double *da, *db, *dc;
  if (dbuf(0, na, &da) || dbuf(1, nb_, &db) || dbuf(2, nc, &dc)) return;
  if (h2d(da, a, na * 8) || h2d(db, b, nb_ * 8)) return;
  if (dev_mxm(da, *n1, db, *n2, dc, *n3, S.s)) return;
  if (d2h(c, dc, nc * 8)) return;
  sync();
}

// ---------------------------------------------------------------- cg.f --
void local_grad3_(double *ur, double *us, double *ut, const double *u,
                  const int *n, const double *D, const double *Dt) {
  clear_status();
  State &S = st();
  if (S.init()) return;
  const int m1 = *n + 1;
  if (m1 < 1 || m1 > 64) {
    fail(NB_ERR_ARG, "local_grad3: n=%d", *n);
    return;
  }
  const long m3 = long(m1) * m1 * m1, m2 = long(m1) * m1;
  double *du, *dr, *ds, *dt, *dD, *dDt;
  if (dbuf(0, m3, &du) || dbuf(1, m3, &dr) || dbuf(2, m3, &ds) ||
      dbuf(3, m3, &dt) || dbuf(4, m2, &dD) || dbuf(5, m2, &dDt))
    return;
  if (h2d(du, u, m3 * 8) || h2d(dD, D, m2 * 8) || h2d(dDt, Dt, m2 * 8)) return;
  if (dev_local_grad3(dr, ds, dt, du, *n, dD, dDt, S.s)) return;
  if (d2h(ur, dr, m3 * 8) || d2h(us, ds, m3 * 8) || d2h(ut, dt, m3 * 8)) return;
  sync();
}

void local_grad3_t_(double *u, const double *ur, const double *us,
                    const double *ut, const int *N, const double *D,
                    const double *Dt, double *w) {
  clear_status();
  State &S = st();
  if (S.init()) return;
  const int m1 = *N + 1;
  if (m1 < 1 || m1 > 64) {
    fail(NB_ERR_ARG, "local_grad3_t: N=%d", *N);
    return;
  }
  const long m3 = long(m1) * m1 * m1, m2 = long(m1) * m1;
  double *du, *dr, *ds, *dt, *dD, *dDt, *dw;
  if (dbuf(0, m3, &du) || dbuf(1, m3, &dr) || dbuf(2, m3, &ds) ||
      dbuf(3, m3, &dt) || dbuf(4, m2, &dD) || dbuf(5, m2, &dDt) || dbuf(6, m3, &dw))
    return;
  if (h2d(dr, ur, m3 * 8) || h2d(ds, us, m3 * 8) || h2d(dt, ut, m3 * 8) ||
      h2d(dD, D, m2 * 8) || h2d(dDt, Dt, m2 * 8))
    return;
  if (dev_local_grad3_t(du, dr, ds, dt, *N, dD, dDt, dw, S.s)) return;
  if (d2h(u, du, m3 * 8) || d2h(w, dw, m3 * 8)) return;
  sync();
}

void ax_e_(double *w, const double *u, const double *g, double *ur,
           double *us, double *ut, double *wk) {
  (void)ur; (void)us; (void)ut; (void)wk;
  clear_status();
  State &S = st();
  if (check_common() || S.init()) return;
  const int lx = S.nx1;
  const long m3 = long(lx) * lx * lx;
  double *dw, *du, *dg, *dD;
  if (dbuf(0, m3, &dw) || dbuf(1, m3, &du) || dbuf(2, 6 * m3, &dg) || dbuf(3, lx * lx, &dD)) return;
  if (h2d(du, u, m3 * 8) || h2d(dg, g, 6 * m3 * 8) || h2d(dD, S.dxm1.data(), lx * lx * 8)) return;
  Operator one;  // no even-odd tables: the reference's left-to-right sums
  one.lx = lx;
  one.nelt = 1;
  one.n = m3;
  AxArgs<double> a{};
  a.w = dw;
  a.u = du;
  a.g = dg;
  a.D = dD;
  if (launch_ax<double>(one, 0, a, S.s)) return;
  if (d2h(w, dw, m3 * 8)) return;
  sync();
}

void ax_(double *w, const double *u, const double *gxyz, double *ur,
         double *us, double *ut, double *wk, const int *n) {
  (void)ur; (void)us; (void)ut; (void)wk;
  clear_status();
  State &S = st();
  Operator *op = nullptr;
  if (common_op(&op)) return;
  if (*n != op->n) {
    fail(NB_ERR_ARG, "ax: n=%d, mesh has %ld points", *n, op->n);
    return;
  }
  const long nn = op->n;
  double *dw, *du, *dg;
  if (dbuf(0, nn, &dw) || dbuf(1, nn, &du) || dbuf(2, 6 * nn, &dg)) return;
  if (h2d(du, u, nn * 8) || h2d(dg, gxyz, 6 * nn * 8)) return;
  metric_fx_invalidate(*op);
  if (apply_ax<double>(*op, dw, du, dg, S.s)) return;
  if (d2h(w, dw, nn * 8)) return;
  if (sync()) return;
  S.flop_a += ax_flops(S.nx1, S.nelt);
}

void maskit_(double *w, double *pmask, const int *nx, const int *ny,
             const int *nz) {
  clear_status();
  State &S = st();
  if (check_common() || S.init()) return;
  const int lx = *nx;
  (void)ny;
  (void)nz;
  const long nxyz = long(lx) * lx * lx, nn = nxyz * S.nelt;
  double *dw;
  if (dbuf(0, nn, &dw)) return;
  if (h2d(dw, w, nn * 8)) return;
  std::vector<int> list;
  if (pmask[0] < 0) {
    const int cnt = int(pmask[1]);
    list.resize(cnt);
    for (int i = 0; i < cnt; ++i) list[i] = int(pmask[2 + i]) - 1;
  } else {
    // build branch: zero all elements' domain faces, record element 1's zeros
    for (int e = 0; e < S.nelt; ++e) {
      const unsigned f = face_bits(S.lglel[e], S.nelx, S.nely, S.nelz);
      for (int k = 0; k < lx; ++k)
        for (int j = 0; j < lx; ++j)
          for (int i = 0; i < lx; ++i) {
            const bool m = ((f & 1u) && i == 0) || ((f & 2u) && i == lx - 1) ||
                           ((f & 4u) && j == 0) || ((f & 8u) && j == lx - 1) ||
                           ((f & 16u) && k == 0) || ((f & 32u) && k == lx - 1);
            if (m) list.push_back(int(nxyz * e + i + lx * j + lx * lx * k));
          }
    }
  }
  int *dl = nullptr;
  if (!list.empty()) {
    if (dbuf(1, list.size(), &dl) || h2d(dl, list.data(), list.size() * 4)) return;
    if (vec_mask<double>(dw, dl, int(list.size()), S.s)) return;
  }
  if (d2h(w, dw, nn * 8) || sync()) return;
  if (pmask[0] >= 0) {
    long nm = 0;
    for (int e = 0; e < S.nelt; ++e)
      for (long i = 0; i < nxyz; ++i)
        if (w[i] == 0) pmask[2 + nm++] = double(i + 1);
    pmask[0] = -1.0;
    pmask[1] = double(nm);
  }
}

void solvem_(double *z, const double *r, const int *n) {
  clear_status();
  State &S = st();
  if (!S.mgrid) {
    std::memcpy(z, r, sizeof(double) * size_t(*n));  // hsmg_dum.f:9-14
    return;
  }
  std::vector<double> rr(r, r + *n);
  h1mg_solve_(z, rr.data(), n);
}

void cg_(double *x, const double *f, const double *g, const double *c,
         double *r, double *w, double *p, double *z, const int *n,
         const int *niter, double *flop_cg) {
  clear_status();
  State &S = st();
  Operator *op = nullptr;
  if (common_op(&op)) return;
  if (*n != op->n) {
    fail(NB_ERR_ARG, "cg: n=%d, mesh has %ld points", *n, op->n);
    return;
  }
  if (*niter < 0) {
    fail(NB_ERR_ARG, "cg: niter=%d", *niter);
    return;
  }
  const long nn = op->n;
  double *dx, *df, *dg, *dc, *dr, *dw, *dp, *dz;
  if (dbuf(0, nn, &dx) || dbuf(1, nn, &df) || dbuf(2, 6 * nn, &dg) ||
      dbuf(3, nn, &dc) || dbuf(4, nn, &dr) || dbuf(5, nn, &dw) ||
      dbuf(6, nn, &dp) || dbuf(7, nn, &dz))
    return;
  if (h2d(df, f, nn * 8) || h2d(dg, g, 6 * nn * 8) || h2d(dc, c, nn * 8)) return;
  std::unique_ptr<MgPrecond> M;
  if (S.mgrid) {
    if (!S.mg) {
      fail(NB_ERR_STATE, "cg: MGRID selected but h1mg_setup_ not called");
      return;
    }
    M.reset(new MgPrecond(S.mg.get()));
  }
  if (cg_device(*op, S.wk, dx, df, dg, dc, dr, dw, dp, dz, *niter, M.get(),
                false, S.s))
    return;
  if (d2h(x, dx, nn * 8) || d2h(r, dr, nn * 8)) return;
  // w, p and z are written only by an iteration (cg.f:48-75); with niter = 0
  // the caller's arrays stay as they were, as in the reference
  if (*niter > 0 &&
      (d2h(w, dw, nn * 8) || d2h(p, dp, nn * 8) || d2h(z, dz, nn * 8)))
    return;
  if (sync() || device_error_check(S.s)) return;
  const int iter = *niter + 1;
  for (int k = 0; k < *niter; ++k) S.flop_a += ax_flops(S.nx1, S.nelt);
  const double inc = double(wrap_mul(wrap_mul(iter, 15), *n));
  *flop_cg = *flop_cg + inc;
  S.flop_cg = *flop_cg;
}

// The values the reference's cg prints (cg.f:44,79): rnorm at iteration 0,
// then the final iteration count (niter+1), rnorm, alpha, beta, pap.
void nekbone_cg_report_(int *iter, double *rnorm0, double *rnorm, double *alpha,
                        double *beta, double *pap) {
  clear_status();
  State &S = st();
  if (!S.wk.sc) {
    fail(NB_ERR_STATE, "nekbone_cg_report: no cg call yet");
    return;
  }
  CgScalars sc;
  if (cudaMemcpyAsync(&sc, S.wk.sc, sizeof(sc), cudaMemcpyDeviceToHost, S.s) != cudaSuccess ||
      cudaStreamSynchronize(S.s) != cudaSuccess) {
    fail(NB_ERR_CUDA, "nekbone_cg_report: reading the solver scalars");
    return;
  }
  // the history rows (rnorm, alpha, beta, pap, rtz1) of iteration 0 and of
  // the last iteration: the scalars themselves already hold the next beta
  double h0[5] = {0, 0, 0, 0, 0}, hl[5] = {sc.rnorm, sc.alpha, sc.beta, sc.pap, sc.rtz1};
  if (S.wk.hist && sc.iter < S.wk.hist_len) {
    if (cudaMemcpyAsync(h0, S.wk.hist, sizeof(h0), cudaMemcpyDeviceToHost, S.s) !=
            cudaSuccess ||
        cudaMemcpyAsync(hl, S.wk.hist + 5 * sc.iter, sizeof(hl), cudaMemcpyDeviceToHost,
                        S.s) != cudaSuccess ||
        cudaStreamSynchronize(S.s) != cudaSuccess) {
      fail(NB_ERR_CUDA, "nekbone_cg_report: reading the iteration history");
      return;
    }
  }
  if (iter) *iter = sc.iter + 1;
  if (rnorm0) *rnorm0 = h0[0];
  if (rnorm) *rnorm = hl[0];
  if (alpha) *alpha = hl[1];
  if (beta) *beta = hl[2];
  if (pap) *pap = hl[3];
}

// -------------------------------------------------------------- hsmg.f --
void h1mg_setup_(void) {
  clear_status();
  State &S = st();
  Operator *op = nullptr;
  if (common_op(&op)) return;
  std::unique_ptr<Multigrid> mg(new Multigrid());
  if (mg_setup(mg.get(), *op, nullptr, 0, S.s)) return;
  S.mg = std::move(mg);
}

void h1mg_solve_(double *z, double *rhs, const int *nn) {
  clear_status();
  State &S = st();
  Operator *op = nullptr;
  if (common_op(&op)) return;
  if (!S.mg) {
    fail(NB_ERR_STATE, "h1mg_solve: h1mg_setup_ not called");
    return;
  }
  if (*nn != op->n) {
    fail(NB_ERR_ARG, "h1mg_solve: n=%d, mesh has %ld points", *nn, op->n);
    return;
  }
  const long n = op->n;
  double *dz, *dr;
  if (dbuf(8, n, &dz) || dbuf(9, n, &dr)) return;
  if (h2d(dr, rhs, n * 8)) return;
  if (mg_solve(*S.mg, dz, dr, S.s)) return;
  if (d2h(z, dz, n * 8) || d2h(rhs, dr, n * 8) || sync()) return;
}

// --------------------------------------------------------- set-up path --
void zwgll_(double *z, double *w, const int *np) { zwgll(z, w, *np); }

void semhat_(double *a, double *b, double *c, double *d, double *z, double *w,
             const int *n) {
  (void)w;
  semhat(a, b, c, d, z, *n);
}

void cubic_(int *mx, int *my, int *mz, const int *np) { cubic(mx, my, mz, *np); }

void get_exyz_(int *ex, int *ey, int *ez, const int *eg, const int *nelx, const int *nely,
               const int *nelz) {
  (void)nelz;  // the reference takes it and does not use it
  get_exyz(ex, ey, ez, *eg, *nelx, *nely);
}

void set_vert_box_(int64_t *glo_num, const int *nx) {
  clear_status();
  State &S = st();
  if (check_common()) return;
  set_vert_box(glo_num, *nx, S.nelt, S.nelx, S.nely, S.lglel.data());
}

// body(lo, hi) over [0, n) split across the host's threads: the set-up
// loops below compute every entry on its own, so the split changes nothing
extern "C++" {
template <typename F>
static void host_parallel(long n, F body) {
  const long nt = std::max(1L, std::min<long>(std::thread::hardware_concurrency(), n / 65536));
  if (nt == 1) {
    body(0L, n);
    return;
  }
  std::vector<std::thread> th;
  for (long t = 0; t < nt; ++t) th.emplace_back(body, n * t / nt, n * (t + 1) / nt);
  for (auto &x : th) x.join();
}
}

void setup_g_(double *g) {
  clear_status();
  State &S = st();
  if (check_common()) return;
  const int lx = S.nx1;
  std::vector<double> a(lx * lx), b(lx), c(lx * lx), d(lx * lx), z(lx);
  semhat(a.data(), b.data(), c.data(), d.data(), z.data(), lx - 1);
  const long l3 = long(lx) * lx * lx;
  host_parallel(long(S.nelt) * l3, [&](long lo, long hi) {
    for (long p = lo; p < hi; ++p) {
      const int r = int(p % l3), i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
      double *gp = g + 6 * p;
      const double v = b[i] * b[j] * b[k];
      gp[0] = v;
      gp[1] = gp[2] = 0.;
      gp[3] = v;
      gp[4] = 0.;
      gp[5] = v;
    }
  });
}

void set_multiplicity_(double *c) {
  clear_status();
  State &S = st();
  if (check_common()) return;
  const long n = long(S.nelt) * S.nx1 * S.nx1 * S.nx1;
  for (long i = 0; i < n; ++i) c[i] = 1.0;
  const int dom = 1, op = 1, tr = 0;
  gs_op_(&S.gsh, c, &dom, &op, &tr);
  if (last_status()) return;
  for (long i = 0; i < n; ++i) c[i] = 1. / c[i];
}

void set_f_(double *f, const double *c, const int *n) {
  clear_status();
  host_parallel(*n, [&](long lo, long hi) {
    for (long q = lo; q < hi; ++q) {
      const int i = int(q + 1);
      double arg = 1.e9 * double(wrap_mul(i, i));
      arg = 1.e9 * std::cos(arg);
      f[q] = std::sin(arg);
    }
  });
  dssum_(f);
  if (last_status()) return;
  for (int i = 0; i < *n; ++i) f[i] = f[i] * c[i];
}

// ------------------------------------------------------------ device API --
int nb_mesh_create(nb_mesh **mesh, int nelx, int nely, int nelz, int lx1,
                   int mask_mode) {
  clear_status();
  if (st().init()) return last_status();
  if (mask_mode != 0 && mask_mode != 1)
    return fail(NB_ERR_ARG, "mask_mode %d not 0 or 1", mask_mode);
  std::unique_ptr<nb_mesh> m(new nb_mesh());
  NB_TRY(operator_box(&m->op, nelx, nely, nelz, lx1, mask_mode, st().s));
  *mesh = m.release();
  return NB_OK;
}

void nb_set_setup_on_device(int on) { set_setup_on_device(on != 0); }
void nb_set_mg_fixed_kernels(int on) { mg_set_fixed_kernels(on != 0); }

int nb_eo_line_maps(int lx1, int *plane, unsigned char *rmap, unsigned char *smap) {
  clear_status();
  int pl = 0;
  switch (lx1) {
    case 2: pl = eo_plane<float, 2>(); break;
    case 4: pl = eo_plane<float, 4>(); break;
    case 6: pl = eo_plane<float, 6>(); break;
    case 8: pl = eo_plane<float, 8>(); break;
    case 10: pl = eo_plane<float, 10>(); break;
    case 12: pl = eo_plane<float, 12>(); break;
    default: return fail(NB_ERR_ARG, "nb_eo_line_maps: lx1=%d (even, 2..12)", lx1);
  }
  if (!rmap || !smap) return fail(NB_ERR_ARG, "nb_eo_line_maps: null map");
  if (plane) *plane = pl;
  eo_line_maps(lx1, pl, rmap, smap);
  return NB_OK;
}

// Copies one device int array (count entries) to host, when dst is given.
static int copy_out(void *dst, const void *src, size_t bytes) {
  if (!dst || !bytes) return NB_OK;
  NB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st().s));
  NB_CUDA(cudaStreamSynchronize(st().s));
  return NB_OK;
}

int nb_mesh_gs_maps(const nb_mesh *mesh, int *ng, long *nmem, int *off, int *idx) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  const GsDevice &g = mesh->op.gs;
  if (!g.symmetric) return fail(NB_ERR_STATE, "nb_mesh_gs_maps: flagged ids (no symmetric map)");
  int end = 0;
  if (g.ng >= 0) NB_TRY(copy_out(&end, g.off + g.ng, sizeof(int)));
  if (ng) *ng = g.ng;
  if (nmem) *nmem = end;
  NB_TRY(copy_out(off, g.off, size_t(g.ng + 1) * sizeof(int)));
  NB_TRY(copy_out(idx, g.idx, size_t(end) * sizeof(int)));
  return NB_OK;
}

int nb_mesh_boundary_groups(const nb_mesh *mesh, int *nbg, long *nmem, int *off,
                            unsigned *idx) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  const Operator &op = mesh->op;
  if (!op.fused_ok || !op.bnd_off) return fail(NB_ERR_STATE, "no fused boundary groups");
  int end = 0;
  NB_TRY(copy_out(&end, op.bnd_off + op.nbg, sizeof(int)));
  if (nbg) *nbg = op.nbg;
  if (nmem) *nmem = end;
  NB_TRY(copy_out(off, op.bnd_off, size_t(op.nbg + 1) * sizeof(int)));
  NB_TRY(copy_out(idx, op.bnd_idx, size_t(end) * sizeof(unsigned)));
  return NB_OK;
}

int nb_mesh_mask_list(const nb_mesh *mesh, int *n, int *list) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (n) *n = mesh->op.n_mask;
  return copy_out(list, mesh->op.d_mask_list, size_t(mesh->op.n_mask) * sizeof(int));
}

int nb_mesh_set_order(nb_mesh *mesh, int order) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (order < 0 || order > 2) return fail(NB_ERR_ARG, "order %d not 0, 1 or 2", order);
  mesh->op.order = order;
  return NB_OK;
}

int nb_mesh_destroy(nb_mesh *mesh) {
  delete mesh;
  return NB_OK;
}

long nb_mesh_npts(const nb_mesh *mesh) { return mesh ? mesh->op.n : 0; }

int nb_mesh_info(const nb_mesh *mesh, int *nelt, int *lx1, int *fused) {
  if (!mesh) return fail(NB_ERR_HANDLE, "nb_mesh_info: null mesh");
  if (nelt) *nelt = mesh->op.nelt;
  if (lx1) *lx1 = mesh->op.lx;
  if (fused) *fused = mesh->op.fused_ok ? 1 : 0;
  return NB_OK;
}

int nb_setup_g(nb_mesh *mesh, double *g) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  NB_TRY(dev_setup_g(mesh->op, g, st().s));
  return NB_OK;
}

int nb_setup_g_deformed(nb_mesh *mesh, double *g, uint64_t seed, double amp) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  return dev_setup_g_deformed(mesh->op, g, seed, amp, st().s);
}

int nb_ax_tc(nb_mesh *mesh, float *w, const float *u, const float *g) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (mesh->op.mask_mode == 0 && !mesh->op.mask_built)
    return fail(NB_ERR_STATE, "nb_ax_tc: the reference mask list is not built yet");
  return apply_ax_tc(mesh->op, w, u, g, st().s);
}

int nb_ax_f32(nb_mesh *mesh, float *w, const float *u, const float *g) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  NB_TRY(apply_ax<float>(mesh->op, w, u, g, st().s));
  return NB_OK;
}

int nb_set_multiplicity(nb_mesh *mesh, double *c) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  const long n = mesh->op.n;
  std::vector<double> one(n, 1.0);
  NB_TRY(h2d(c, one.data(), n * 8));
  NB_TRY(gs_exec(mesh->op.gs, c, 1, 1, 0, st().s));
  NB_TRY(sync());
  std::vector<double> h(n);
  NB_TRY(d2h(h.data(), c, n * 8));
  NB_TRY(sync());
  for (long i = 0; i < n; ++i) h[i] = 1. / h[i];
  NB_TRY(h2d(c, h.data(), n * 8));
  return sync();
}

int nb_rhs_uniform(nb_mesh *mesh, double *f, const double *c, uint64_t seed) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  NB_TRY(dev_rhs_uniform(mesh->op, f, c, seed, st().s));
  return sync();
}

int nb_ax(nb_mesh *mesh, double *w, const double *u, const double *g) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  metric_fx_invalidate(mesh->op);
  NB_TRY(apply_ax<double>(mesh->op, w, u, g, st().s));
  return NB_OK;
}

int nb_dssum(nb_mesh *mesh, void *u, int dom) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  return gs_exec(mesh->op.gs, u, dom, 1, 0, st().s);
}

int nb_cg(nb_mesh *mesh, double *x, const double *f, const double *g,
          const double *c, double *r, double *w, double *p, double *z,
          int niter, int flags, double *hist) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  std::unique_ptr<MgPrecond> M;
  if (flags & 2) {
    if (!mesh->mg) {
      std::unique_ptr<Multigrid> mg(new Multigrid());
      NB_TRY(mg_setup(mg.get(), mesh->op, nullptr, 0, st().s));
      mesh->mg = std::move(mg);
    }
    M.reset(new MgPrecond(mesh->mg.get()));
  }
  NB_TRY(cg_device(mesh->op, mesh->wk, x, f, g, c, r, w, p, z, niter, M.get(),
                   (flags & 1) != 0, st().s));
  if (hist) {
    NB_TRY(d2h(hist, mesh->wk.hist, sizeof(double) * 5 * (niter + 1)));
    NB_TRY(sync());
  }
  return NB_OK;
}

int nb_cg_f32(nb_mesh *mesh, float *x, const float *f, const float *g,
              const float *c, float *r, float *w, float *p, int niter,
              double *hist) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  NB_TRY(cg_device_f32(mesh->op, mesh->wk, x, f, g, c, r, w, p, niter, st().s));
  if (hist) {
    NB_TRY(d2h(hist, mesh->wk.hist, sizeof(double) * 5 * (niter + 1)));
    NB_TRY(sync());
  }
  return NB_OK;
}

int nb_mesh_parts(nb_mesh *mesh, void **op, void **wk) {
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  *op = &mesh->op;
  *wk = &mesh->wk;
  return NB_OK;
}

void *nb_stream(void) { return (void *)lib_stream(); }

int nb_time_cg_kernels(nb_mesh *mesh, double *x, const double *f,
                       const double *g, const double *c, double *r, double *w,
                       double *p, int reps, double *ms3) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (!mesh->op.fused_ok) return fail(NB_ERR_UNSUPPORTED, "mesh has no fused path");
  return time_cg_kernels_t<double>(mesh->op, mesh->wk, x, f, g, c, r, w, p, reps,
                                   ms3, lib_stream());
}

int nb_time_cg_kernels_f32(nb_mesh *mesh, float *x, const float *f,
                           const float *g, const float *c, float *r, float *w,
                           float *p, int reps, double *ms3) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (!mesh->op.fused_ok) return fail(NB_ERR_UNSUPPORTED, "mesh has no fused path");
  return time_cg_kernels_t<float>(mesh->op, mesh->wk, x, f, g, c, r, w, p, reps,
                                  ms3, lib_stream());
}

int nb_mg_setup(nb_mesh *mesh, const int *orders, int nlev, int precision) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  std::unique_ptr<Multigrid> mg(new Multigrid());
  NB_TRY(mg_setup(mg.get(), mesh->op, orders, nlev, st().s, precision));
  mesh->mg = std::move(mg);
  return NB_OK;
}

int nb_mg_setup_coarse(nb_mesh *mesh, const double *g) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (!mesh->mg) return fail(NB_ERR_STATE, "nb_mg_setup_coarse: call nb_mg_setup first");
  return mg_setup_coarse(mesh->mg.get(), g, st().s);
}

int nb_mg_solve(nb_mesh *mesh, double *z, double *rhs) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (!mesh->mg) return fail(NB_ERR_STATE, "nb_mg_solve: call nb_mg_setup first");
  return mg_solve(*mesh->mg, z, rhs, st().s);
}

int nb_pcg_tol(nb_mesh *mesh, double *x, const double *f, const double *g,
               const double *c, double tol, int max_iter, int check_every,
               int *iters, double *relres) {
  clear_status();
  if (!mesh) return fail(NB_ERR_HANDLE, "null mesh");
  if (!mesh->mg) return fail(NB_ERR_STATE, "nb_pcg_tol: call nb_mg_setup first");
  cudaStream_t s = lib_stream();
  Operator &op = mesh->op;
  CgWork &wk = mesh->wk;
  const long n = op.n;
  if (check_every < 1) check_every = 1;
  NB_TRY(wk.ensure_scratch(size_t(4) * n * 8));
  double *r = reinterpret_cast<double *>(wk.scratch);
  double *w = r + n, *p = w + n, *z = p + n;
  MgPrecond M(mesh->mg.get());
  int done = 0, stt = NB_OK;
  double rn0 = 0.0, rn = 0.0;
  stt = cg_begin(op, wk, x, f, c, r, max_iter, s);
  if (!stt && cudaMemcpy(&rn0, &wk.sc->rnorm, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
    stt = fail(NB_ERR_CUDA, "nb_pcg_tol: reading rnorm");
  rn = rn0;
  while (!stt && done < max_iter) {
    const int k = std::min(check_every, max_iter - done);
    stt = cg_steps_pc(op, wk, x, g, c, r, w, p, z, done + 1, done + k, &M, s);
    done += k;
    if (!stt && (cudaMemcpyAsync(&rn, &wk.sc->rnorm, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                 cudaStreamSynchronize(s) != cudaSuccess))
      stt = fail(NB_ERR_CUDA, "nb_pcg_tol: reading rnorm");
    if (rn0 > 0 && rn / rn0 <= tol) break;
  }
  if (stt) return stt;
  NB_TRY(device_error_check(s));
  if (iters) *iters = done;
  if (relres) *relres = rn0 > 0 ? rn / rn0 : 0.0;
  return NB_OK;
}

int nb_sync(void) {
  clear_status();
  if (st().init()) return last_status();
  NB_TRY(sync());
  return device_error_check(st().s);
}

}  // extern "C"

/*
 * nb_oracle.h -- CPU restatement of the Nekbone spectral-element Poisson CG
 * hot path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * bench.py CPU-baseline / reference arm may load this library, and only as the
 * checker or as the timed CPU baseline.  The product (nekbone_gb300) never
 * links, loads or calls it.
 *
 * Parity status:
 *   - gather-scatter (orc_gs_*): pinned bit-exactly against the reference's
 *     own jl library (src/jl/gs.c, src/jl/gs_local.c) compiled from the
 *     reference sources into oracle/_ref/ by oracle/Makefile, and against the
 *     known answers of src/jl/gs_test.c.
 *   - everything restated from the Fortran sources -- GLL points, semhat,
 *     cubic, set_vert_box, setup_g, set_multiplicity, set_f, ax with the
 *     reference's maskit, the driver's two cg calls with every glsc3 value,
 *     and hsmg: pinned against golden vectors from the reference's own
 *     Fortran sources executed by oracle/f77.py, a Fortran 77 subset
 *     executor (no Fortran compiler exists in this image), with the
 *     reference's jl library for gather-scatter
 *     (tests/golden/make_golden_fortran.py).  The plain build (ORC_FMA=0)
 *     reproduces them bit for bit, including the C1 configuration (4^3
 *     elements, lx1=10, 2 x 100 iterations).  hsmg agrees to 1e-12: its
 *     generalised eigenproblems are solved by a different eigensolver
 *     (Jacobi here, LAPACK dsygv there).
 *
 * Arrays follow the reference's Fortran layout (column-major, element-major,
 * i fastest) with 0-based C indexing.
 */
#ifndef NB_ORACLE_H
#define NB_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- speclib.f / semhat.f ------------------------------------------------ */
void   orc_zwgljd(double *z, double *w, int np, double alpha, double beta);
void   orc_zwgll(double *z, double *w, int np);
void   orc_fd_weights_full(double xx, const double *x, int n, int m, double *c);
void   orc_semhat(double *a, double *b, double *c, double *d, double *z, int n);

/* ---- driver.f / prox_dssum.f ---------------------------------------------- */
void    orc_cubic(int *mx, int *my, int *mz, int np);
/* init_mesh for np=1, nid=0; fills nelx/nely/nelz and lglel[nelt] (1-based ids) */
void    orc_init_mesh(int ifbrick, int nelt, int mx, int my, int mz,
                      int *nelx, int *nely, int *nelz, int *lglel);
void    orc_set_vert_box(int64_t *glo_num, int nx, int nelt, int nelx,
                         int nely, int nelz, const int *lglel);

/* ---- jl gather-scatter restatement ---------------------------------------- */
typedef struct orc_gs orc_gs;
orc_gs *orc_gs_setup(const int64_t *ids, int n);
void    orc_gs_free(orc_gs *h);
/* dom: 1 double, 2 float, 3 int, 4 long(int64); op: 1 add, 2 mul, 3 min, 4 max */
void    orc_gs_op(const orc_gs *h, void *u, int dom, int op, int transpose);
/* expose the local maps: which 0 = unflagged, 1 = all, 2 = flagged primaries */
int     orc_gs_map_len(const orc_gs *h, int which);
void    orc_gs_map_copy(const orc_gs *h, int which, uint32_t *out);

/* ---- the solver context (mirrors the reference's common blocks) ----------- */
typedef struct orc_ctx orc_ctx;
/* mask_mode: 0 = reference maskit (element-1 quirk), 1 = full Dirichlet mask */
orc_ctx *orc_ctx_new(int nelx, int nely, int nelz, int nelt, int nx1,
                     const int *lglel, int mask_mode, int nthreads);
void     orc_ctx_free(orc_ctx *c);
void     orc_ctx_set_threads(orc_ctx *c, int nthreads);
void     orc_ctx_reset_mask(orc_ctx *c);            /* init_mesh: cmask(-1)=1 */
int      orc_ctx_n(const orc_ctx *c);
const double *orc_ctx_dxm1(const orc_ctx *c);
const double *orc_ctx_wxm1(const orc_ctx *c);
const double *orc_ctx_zgm1(const orc_ctx *c);
void     orc_setup_g(const orc_ctx *c, double *g);       /* prox_setup.f:27 */
void     orc_set_multiplicity(orc_ctx *c, double *mult); /* driver.f:274  */
void     orc_set_f(orc_ctx *c, double *f, const double *mult); /* driver.f:88 */
void     orc_dssum(orc_ctx *c, double *f);
void     orc_maskit(orc_ctx *c, double *w);

/* ---- math.f / mxm --------------------------------------------------------- */
void   orc_mxm(const double *a, int n1, const double *b, int n2, double *c,
               int n3);
double orc_glsc3(const double *a, const double *b, const double *mult, int n);
void   orc_add2s1(double *a, const double *b, double c1, int n);
void   orc_add2s2(double *a, const double *b, double c1, int n);

/* ---- cg.f ----------------------------------------------------------------- */
void orc_local_grad3(double *ur, double *us, double *ut, const double *u,
                     int n, const double *D, const double *Dt);
void orc_local_grad3_t(double *u, const double *ur, const double *us,
                       const double *ut, int n, const double *D,
                       const double *Dt, double *w);
void orc_ax_e(orc_ctx *c, double *w, const double *u, const double *g);
/* w = mask(QQ^T A_L u + 0.1 u); element-local product only when full==0 */
void orc_ax(orc_ctx *c, double *w, const double *u, const double *g);
void orc_ax_local(orc_ctx *c, double *w, const double *u, const double *g);
/* cg: fixed niter iterations; hist (optional, 5*(niter+1)) receives
 * rnorm,alpha,beta,pap,rtz1 per iteration (index 0 = initial rnorm).
 * use_mg: 0 = identity preconditioner (hsmg_dum.f), 1 = h1mg_solve. */
int  orc_cg(orc_ctx *c, double *x, const double *f, const double *g,
            const double *mult, double *r, double *w, double *p, double *z,
            int n, int niter, int use_mg, double *hist);
double orc_flop_a(const orc_ctx *c);
double orc_flop_cg(const orc_ctx *c);

/* ---- hsmg.f --------------------------------------------------------------- */
/* levels: NULL = the reference's level choice (h1mg_setup_mg_nx);
 * otherwise nlev polynomial orders, coarsest first. */
int  orc_h1mg_setup(orc_ctx *c, const int *orders, int nlev);
void orc_h1mg_solve(orc_ctx *c, double *z, double *rhs, int n);
int  orc_h1mg_nlev(const orc_ctx *c);
int  orc_h1mg_order(const orc_ctx *c, int l);    /* l = 1..nlev */
/* FDM data of level l (2..nlev): s (nl*nl*2*3*nelt), d (nl^3*nelt) */
void orc_h1mg_fdm_copy(const orc_ctx *c, int l, double *s, double *d);
/* generalized symmetric eigenproblem A x = lam B x (dsygv itype 1, 'V') */
int  orc_generalev(double *a, double *b, double *lam, int n);

/* ---- fp-contraction variant this library was built with ------------------- */
int  orc_fma_variant(void);

#ifdef __cplusplus
}
#endif
#endif

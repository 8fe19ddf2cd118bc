/*
 * nekbone_gb300.h -- C ABI of the GB300 implementation of Nekbone's
 * spectral-element Poisson CG hot path.
 *
 * Two layers:
 *
 *  1. Drop-in entry points with the reference's Fortran calling convention
 *     (lower case, trailing underscore, every argument by reference, REAL =
 *     double, INTEGER = int32_t, global ids int64_t).  They take HOST arrays,
 *     exactly as the Fortran driver passes them, move them to the GPU, run the
 *     CUDA kernels and copy the results back.  Each declaration cites the
 *     reference routine it replaces (file:line in the reference project).
 *     Routines that read Fortran common blocks in the reference read the
 *     values published by nekbone_common_ here.
 *
 *  2. A device-resident API (nb_*) for callers that keep their vectors on the
 *     GPU: mesh construction, ax, gather-scatter and the CG solvers on device
 *     pointers, with no host round trip inside a solve.
 *
 * Errors: every call records a status (0 = ok).  In the default error mode
 * (0) a failing call prints its message and exits the process with status 1,
 * as the reference's jl fail() does (jl/fail.c:11-52).  In mode 1 the call
 * returns and the status is read with nekbone_last_status().
 */
#ifndef NEKBONE_GB300_H
#define NEKBONE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status -- */
int         nekbone_last_status(void);
const char *nekbone_last_message(void);
void        nekbone_clear_status(void);
/* 0 = reference behaviour (print, exit(1)); 1 = record and return */
void        nekbone_set_error_mode(int mode);
int         nekbone_version(void);

/* ------------------------------------------- common-block publication -- */
/* The Fortran routines below read /dimn/ (SIZE), /hcglb/ lglel (PARALLEL),
 * /dxyz/ dxm1 (DXYZ) and /comm_handles/ gsh (PARALLEL) instead of taking
 * them as arguments.  The Fortran side publishes them once per mesh, after
 * init_mesh, proxy_setupds and proxy_setup (driver.f:43-47). */
void nekbone_common_(const int *nelx, const int *nely, const int *nelz,
                     const int *nelt, const int *nx1, const int *lglel,
                     const double *dxm1, const int *gsh);
/* init_mesh's "cmask(-1) = 1.0" (driver.f:125): the next maskit rebuilds
 * its index list (cg.f:231-254). */
void nekbone_mask_reset_(void);
/* 0 = the reference's maskit (list of element 1's Dirichlet points after the
 * first call, cg.f:224-229); 1 = every element's Dirichlet faces. */
void nekbone_set_mask_mode_(const int *mode);
/* .true. selects h1mg_solve as solveM (MGRID build, cg.f:86-94,
 * hsmg.f:960); .false. the copy of hsmg_dum.f:9-14. */
void nekbone_set_mgrid_(const int *ifmgrid);
/* Form of the FP64 element operator: 0 = the reference's left-to-right mxm
 * sums (mxm_std.f:255; bit-identical to a left-to-right fma evaluation),
 * 1 = even-odd split of the anti-centrosymmetric GLL derivative on the FP64
 * pipe (same result to rounding, ~27% fewer FP64 operations), 2 = the
 * even-odd form in 64-bit fixed point on the integer pipes (default: block
 * floating point, ~55 significant bits of each element's largest value;
 * same result to rounding, ~4x faster on GB300, whose FP64 pipe runs at
 * 1/64 of its FP32 rate).  Odd lx1 falls back to order 0; ax_e_ always uses
 * order 0. */
void nekbone_set_contraction_order_(const int *order);
/* /cflops/ flop_a, flop_cg (INPUT:8), accumulated as the reference does */
void nekbone_get_flops_(double *flop_a, double *flop_cg);
void nekbone_set_flops_(const double *flop_a, const double *flop_cg);

/* What the last cg_ would print (cg.f:44,79): *iter = niter+1, rnorm at
 * iteration 0 and at the end, and the last alpha, beta and pap. */
void nekbone_cg_report_(int *iter, double *rnorm0, double *rnorm, double *alpha,
                        double *beta, double *pap);

/* --------------------------------------- jl gather-scatter (jl/gs.c) -- */
/* gs_setup_ (jl/gs.c:1160-1170).  comm/np are accepted for signature
 * compatibility; one process (np == 1) is supported. */
void gs_setup_(int *handle, const int64_t *glo_num, const int *n,
               const int *comm, const int *np);
/* gs_op_ (jl/gs.c:1188-1193): dom 1 double, 2 float, 3 int, 4 long (64-bit);
 * op 1 add, 2 mul, 3 min, 4 max; transpose != 0 swaps gather/scatter maps. */
void gs_op_(const int *handle, void *u, const int *dom, const int *op,
            const int *transpose);
/* gs_free_ (jl/gs.c:1237-1242); handles are not reused */
void gs_free_(const int *handle);
/* dssum (prox_dssum.f:2-12): gs_op(gsh, f, 1, 1, 0) on the published gsh */
void dssum_(double *f);

/* -------------------------------------------------------- math.f / mxm -- */
/* glsc3 (math.f:603-617): sum a*b*mult */
double glsc3_(const double *a, const double *b, const double *mult,
              const int *n);
/* add2s1 (math.f:534-541): a = c1*a + b */
void add2s1_(double *a, const double *b, const double *c1, const int *n);
/* add2s2 (math.f:544-551): a = a + c1*b */
void add2s2_(double *a, const double *b, const double *c1, const int *n);
/* mxm (mxm_wrapper.f:1-52): c(n1,n3) = a(n1,n2) b(n2,n3) */
void mxm_(const double *a, const int *n1, const double *b, const int *n2,
          double *c, const int *n3);

/* ---------------------------------------------------------------- cg.f -- */
/* cg (cg.f:2-84): niter CG iterations on A = mask(QQ^T A_L + 0.1 I) */
void cg_(double *x, const double *f, const double *g, const double *c,
         double *r, double *w, double *p, double *z, const int *n,
         const int *niter, double *flop_cg);
/* ax (cg.f:96-125): w = mask(QQ^T A_L u + 0.1 u); ur..wk are scratch */
void ax_(double *w, const double *u, const double *gxyz, double *ur,
         double *us, double *ut, double *wk, const int *n);
/* ax_e (cg.f:142-168): one element, w = A_L u */
void ax_e_(double *w, const double *u, const double *g, double *ur,
           double *us, double *ut, double *wk);
/* local_grad3 (cg.f:170-187) */
void local_grad3_(double *ur, double *us, double *ut, const double *u,
                  const int *n, const double *D, const double *Dt);
/* local_grad3_t (cg.f:189-212) */
void local_grad3_t_(double *u, const double *ur, const double *us,
                    const double *ut, const int *N, const double *D,
                    const double *Dt, double *w);
/* maskit (cg.f:214-258); pmask[0] is pmask(-1), pmask[1] is pmask(0) */
void maskit_(double *w, double *pmask, const int *nx, const int *ny,
             const int *nz);
/* solveM (cg.f:86-94) */
void solvem_(double *z, const double *r, const int *n);

/* -------------------------------------------------------------- hsmg.f -- */
/* h1mg_setup (hsmg.f:3-29) on the published mesh */
void h1mg_setup_(void);
/* h1mg_solve (hsmg.f:960-1034); like the reference it masks rhs in place */
void h1mg_solve_(double *z, double *rhs, const int *nn);

/* ------------------------------------- set-up routines on the hot path -- */
/* zwgll (speclib.f:107-122) */
void zwgll_(double *z, double *w, const int *np);
/* semhat (semhat.f:2-37); w is scratch of 2n+2 */
void semhat_(double *a, double *b, double *c, double *d, double *z,
             double *w, const int *n);
/* set_vert_box (prox_dssum.f:42-73) on the published mesh */
void set_vert_box_(int64_t *glo_num, const int *nx);
/* cubic (driver.f:196-247) */
void cubic_(int *mx, int *my, int *mz, const int *np);
/* get_exyz (prox_dssum.f:75-86): brick position (1-based) of global
 * element eg in a nelx x nely x nelz box. */
void get_exyz_(int *ex, int *ey, int *ez, const int *eg, const int *nelx, const int *nely,
               const int *nelz);
/* setup_g (prox_setup.f:27-52) on the published mesh */
void setup_g_(double *g);
/* set_multiplicity (driver.f:274-291) on the published gsh */
void set_multiplicity_(double *c);
/* set_f (driver.f:88-101) */
void set_f_(double *f, const double *c, const int *n);

/* ------------------------------------------ device-resident API (nb_*) -- */
typedef struct nb_mesh nb_mesh;

/* Box mesh nelx*nely*nelz, lx1 points per direction, brick element order
 * and numbering of the reference (driver.f:117-194, prox_dssum.f:42-73).
 * mask_mode 1 = Dirichlet on every outer face. */
int  nb_mesh_create(nb_mesh **mesh, int nelx, int nely, int nelz, int lx1,
                    int mask_mode);
int  nb_mesh_destroy(nb_mesh *mesh);
/* Where box topologies are built: 1 (default) on the device, without a sort
 * (closed-form copies of each box point, jl's group and member order); 0 on
 * the host with jl's sort-based construction (gs_setup, jl/gs.c:88-113,
 * 330-357).  Both give identical maps.  It covers nb_mesh_create and
 * gs_setup_, which recognises set_vert_box's numbering of a brick box (a
 * device check of every point) and otherwise sorts on the host. */
void nb_set_setup_on_device(int on);
/* hsmg kernels: 1 (default) the FDM and inter-level transfer kernels built
 * for fixed sizes where one exists, 0 the general kernels only.  Both make
 * the same sums in the same order (bitwise-equal results). */
void nb_set_mg_fixed_kernels(int on);
/* Mixed solver: 1 (default) when every element's FP32 metric block equals
 * element 0's (a box of equal elements, as setup_g makes), the inner
 * operator reads that one block instead of each element's; 0 always reads
 * each element's.  Same values either way (bitwise-equal results). */
void nb_set_shared_metric(int on);
/* Mixed solver: 1 takes the inner FP32 CG's element products on the tensor
 * cores (nb_ax_tc's operator: FP16 hi+lo split operands, FP32
 * accumulation), each iteration unfused (operator, gather-scatter, dot
 * products, update); 0 (default) the fused CUDA-core iteration.  The FP64
 * defect correction is the same either way, so both reach the tolerance. */
void nb_set_mixed_tensor_cores(int on);
/* CG (cg_, nb_cg: the fused FP64 iteration without preconditioner), the
 * mixed solver's inner FP32 CG and the batched solve's inner CG: 1
 * (default) keeps the search directions in two buffers, odd and even
 * iterations alternating, and updates x once per two iterations (x += a_k
 * p_k, then x += a_k+1 p_k+1, in one pass; the last direction is copied to
 * the caller's p; a batched problem whose inner CG stops mid-pair gets the
 * deferred update before its defect); 0 one direction buffer and an x
 * update every iteration.  The same fused multiply-adds in the same order
 * either way (bitwise-equal results); the first form reads and writes x
 * half as often and takes n more values of device memory.  A batch's
 * graph is rebuilt when the switch changes. */
void nb_set_paired_update(int on);
/* Mixed solver and batched solve: 1 (default) checks whether the FP32 copy
 * of c is, bitwise at every point, a box mesh's inverse multiplicity (2^-m,
 * m the number of the point's extreme local indices on element faces with
 * a neighbour; even lx1 from 4 to 16) -- once per mixed solve, once per
 * nb_batch_setup -- and if so the inner CG's fused iteration forms c
 * instead of reading it (4 bytes a point less in the update, the
 * interior's c = 1 not read by the operator); 0 always reads c.  The same
 * values either way (bitwise-equal results). */
void nb_set_mixed_closed_multiplicity(int on);
/* The mesh's gather-scatter groups (jl order: groups by primary, members
 * ascending) as CSR: *ng groups, *nmem members; off (ng+1) and idx (nmem)
 * are filled when given. */
int nb_mesh_gs_maps(const nb_mesh *mesh, int *ng, long *nmem, int *off, int *idx);
/* The fused pass's element-boundary groups (singletons included), members
 * on a domain face flagged in bit 31. */
int nb_mesh_boundary_groups(const nb_mesh *mesh, int *nbg, long *nmem, int *off,
                            unsigned *idx);
/* The mesh's masked local indices (ascending). */
int nb_mesh_mask_list(const nb_mesh *mesh, int *n, int *list);
/* The FP32 even-odd operator's line order for lx1 (even, 2..12): the r-line
 * (j + lx1 k) and s-line (i + lx1 k) that thread t of the lx1^2-thread CTA
 * takes, dealt so that each warp's lines start in distinct shared-memory
 * banks where the counts allow; *plane = the layout's plane stride in words
 * (rows are lx1 words).  rmap and smap hold lx1^2 entries. */
int nb_eo_line_maps(int lx1, int *plane, unsigned char *rmap, unsigned char *smap);
/* contraction order of this mesh's FP64 operator (see
 * nekbone_set_contraction_order_) */
int  nb_mesh_set_order(nb_mesh *mesh, int order);
long nb_mesh_npts(const nb_mesh *mesh);
int  nb_mesh_info(const nb_mesh *mesh, int *nelt, int *lx1, int *fused);

/* Device vectors (all pointers below are device pointers of length n, or 6n
 * for g).  g = setup_g form; c = inverse multiplicity; f = seeded uniform
 * [-1,1] per global point, dssum'd, times c, masked. */
int nb_setup_g(nb_mesh *mesh, double *g);
int nb_set_multiplicity(nb_mesh *mesh, double *c);
/* Geometric factors of the box with every element the trilinear image of
 * its vertices, each vertex displaced by amp*h*sum_{q<4} a_q sin(k_q.X +
 * phi_q) (h = 2, the reference element's size; mode parameters from
 * splitmix64(seed)).  No counterpart in the reference, whose elements are
 * undeformed (prox_setup.f:27-52). */
int nb_setup_g_deformed(nb_mesh *mesh, double *g, uint64_t seed, double amp);
int nb_rhs_uniform(nb_mesh *mesh, double *f, const double *c, uint64_t seed);

/* w = A u on the device (FP64) */
int nb_ax(nb_mesh *mesh, double *w, const double *u, const double *g);
/* w = A u with the FP32 operator (FP32 u, w and g of 6n floats) */
int nb_ax_f32(nb_mesh *mesh, float *w, const float *u, const float *g);
/* The same with the six derivative contractions on the tcgen05 tensor
 * cores: lines of each element as rows of K-major FP16 tiles, scaled to unit
 * maximum and split hi + lo, three MMAs per tile (hi*hi + hi*lo + lo*hi)
 * accumulated in FP32; metric and sums in FP32 on CUDA cores. */
int nb_ax_tc(nb_mesh *mesh, float *w, const float *u, const float *g);
/* dssum on a device vector (dom 1 double, 2 float) */
int nb_dssum(nb_mesh *mesh, void *u, int dom);

/* Plain FP64 CG, niter iterations (cg.f:2-84), device pointers.  hist
 * (host, may be NULL) receives 5*(niter+1) values per iteration: rnorm,
 * alpha, beta, pap, rtz1.  flags bit0: force the unfused path; bit1: use
 * the hsmg preconditioner (nb_mg_setup first). */
int nb_cg(nb_mesh *mesh, double *x, const double *f, const double *g,
          const double *c, double *r, double *w, double *p, double *z,
          int niter, int flags, double *hist);

/* FP32 CG on device float vectors (the inner solver of the mixed path) */
int nb_cg_f32(nb_mesh *mesh, float *x, const float *f, const float *g,
              const float *c, float *r, float *w, float *p, int niter,
              double *hist);

/* Mixed precision: FP32 inner CG (inner_iters per correction) inside an
 * FP64 defect-correction loop until sqrt(r'Cr)/sqrt(r0'Cr0) <= tol or
 * max_outer corrections.  Returns outer steps in *outer, inner iterations
 * in *inner_total and the final relative residual in *relres. */
int nb_cg_mixed(nb_mesh *mesh, double *x, const double *f, const double *g,
                const double *c, double tol, int inner_iters, int max_outer,
                int *outer, int *inner_total, double *relres);

/* FP64 CG until sqrt(r'Cr)/sqrt(r0'Cr0) <= tol (max_iter cap); checks the
 * residual every check_every iterations. */
int nb_cg_tol(nb_mesh *mesh, double *x, const double *f, const double *g,
              const double *c, double tol, int max_iter, int check_every,
              int *iters, double *relres);

/* glsc3 on device vectors that allocates nothing -- no counterpart in the
 * reference.  For callers that cannot call cudaMalloc while they run: codes
 * whose device memory belongs to their own pool (an OpenACC or CUDA Fortran
 * host), or loops that must not pay cudaMalloc's implicit device
 * synchronisation.  a, b, mult: device vectors of length n; result: one
 * device double, written asynchronously on stream (a cudaStream_t, NULL =
 * the legacy default stream).  The reduction's partial sums live in a fixed
 * device array of the library (about 128 KiB per GPU that loads it, held
 * until exit), so n must not exceed NB_NOALLOC_MAX_N.  Calls share that
 * array: calls that overlap on the GPU race.  The first call on a device
 * looks the array up and launches the kernel for the first time, and with
 * lazy module loading (CUDA's default) that first launch may itself
 * allocate and synchronise: make one warm-up call per device before the
 * region that must not allocate, and before any stream capture. */
#define NB_NOALLOC_MAX_N 67108864L
int nb_glsc3_noalloc(const double *a, const double *b, const double *mult,
                     long n, double *result, void *stream);

/* hsmg on the device mesh.  orders: nlev polynomial orders, coarsest first,
 * the last lx1-1 (NULL = the reference's level choice, hsmg.f:45-97, lx1 <=
 * 10).  precision 64 = FP64 throughout (h1mg_solve's arithmetic); 32 = the
 * Schwarz smoother, restriction and interpolation in FP32, the coarse solve
 * in FP64. */
int nb_mg_setup(nb_mesh *mesh, const int *orders, int nlev, int precision);
/* z = M^-1 rhs (h1mg_solve, hsmg.f:960-1034); masks rhs in place */
/* Replaces the coarse "solve" of the V-cycle (a copy plus dssum in the
 * reference, hsmg.f:945-957) by an exact FP64 solve of the Galerkin coarse
 * operator R A P on the unmasked vertices, for the metric g: the V-cycle's
 * own restriction and interpolation chain around the FP64 operator, probed
 * with 27 colourings of the vertex grid, checked and densely inverted.  Box
 * meshes, mask_mode 1, the coarsest level of order 1, at most 16384 coarse
 * unknowns.  No counterpart in the reference. */
int nb_mg_setup_coarse(nb_mesh *mesh, const double *g);
int nb_mg_solve(nb_mesh *mesh, double *z, double *rhs);
/* FP64 CG preconditioned with the mesh's hsmg until
 * sqrt(r'Cr)/sqrt(r0'Cr0) <= tol (max_iter cap; residual polled every
 * check_every iterations). */
int nb_pcg_tol(nb_mesh *mesh, double *x, const double *f, const double *g,
               const double *c, double tol, int max_iter, int check_every,
               int *iters, double *relres);

/* Self-test of the tensor-core (tcgen05) building blocks: one 128x16x16
 * MMA of small integers (bf16 != 0: BF16 operands, else F16) compared with
 * the exact product; *mismatches = number of wrong results (0 = pass). */
int nb_tc_selftest(int bf16, int *mismatches);

/* Self-test of the bounded waits: one warp waits on an mbarrier that nothing
 * arrives on, giving up after `polls` polls (1..65536) as every wait in the
 * library's kernels gives up after its limit.  Returns the status such a
 * timeout produces (NB_ERR_CUDA, "a device-side wait timed out") and clears
 * the device error word, so the next call runs normally. */
int nb_wait_selftest(unsigned polls);

/* Timeout self-test inside the real kernels: while on (on != 0), every
 * element kernel that brings its metric block in by a bulk copy (the FP32
 * operators with per-element metrics, the batched FP32 operator) sets its
 * barrier to expect 16 bytes more than the copy brings, so its bounded wait
 * runs out for certain.  The CTA then lets the copy land, skips the
 * element's arithmetic and stores, and sets the device error word.  Takes
 * effect for launches enqueued (and batch graphs built) after the call.
 * Results computed meanwhile are invalid; the synchronising calls report
 * NB_ERR_CUDA ("a device-side wait timed out") once and clear the word.
 * Timeouts are reported by nb_sync, cg_, nb_cg_tol, nb_cg_mixed, nb_pcg_tol,
 * nb_batch_result and nb_batch_cycles; the asynchronous calls (nb_ax,
 * nb_ax_f32, nb_ax_tc, nb_cg, nb_batch_solve) leave them to the next of
 * those.  No counterpart in the reference. */
int nb_set_wait_test(int on);

/* Issue rates of the pipes the element operators use, measured on the
 * current device: rates[0] FP64 fused multiply-adds, rates[1] 32x32->64-bit
 * integer multiply-adds (mad.wide.s32), rates[2] 32-bit integer adds,
 * rates[3] FP32 fused multiply-adds, each in operations per second (about
 * 50 ms).  No counterpart in the reference. */
int nb_pipe_rates(double *rates);

/* Synchronise the library's stream. */
int nb_sync(void);
/* The CUDA stream (cudaStream_t) every nb_* and drop-in call runs on, for
 * callers that record events or order their own work against the library. */
void *nb_stream(void);
/* Average device time (ms) of each kernel of one fused FP64 CG iteration --
 * [0] element operator + direction update, [1] boundary gather-scatter and
 * pap, [2] x/r update and rtr -- over reps iterations (over 2 reps with
 * the paired x update of nb_set_paired_update, its two update forms
 * averaged), timed with CUDA events on the library stream.  Vectors as for nb_cg; x
 * and r are overwritten. */
int nb_time_cg_kernels(nb_mesh *mesh, double *x, const double *f,
                       const double *g, const double *c, double *r, double *w,
                       double *p, int reps, double *ms3);
/* The same for the FP32 iteration of the mixed solver's inner CG (float
 * device vectors, g as 6n floats; c formed in closed form when it verifies,
 * as the inner CG does). */
int nb_time_cg_kernels_f32(nb_mesh *mesh, float *x, const float *f,
                           const float *g, const float *c, float *r, float *w,
                           float *p, int reps, double *ms3);

/* ------------------------------------------- batched solves (nb_batch_*) --
 * Many independent box-mesh Dirichlet Poisson problems of uneven element
 * counts and orders (lx1 in {4, 6, 8, 10, 12}), solved together by the
 * mixed solver (FP32 inner CG inside FP64 defect correction) as one CUDA
 * graph launch.  No counterpart in the reference, which solves one mesh per
 * process (driver.f:42-59); each problem is the mesh nb_mesh_create builds
 * with mask_mode 1, and its vectors live at nb_batch_problem's offset in the
 * batch's concatenated device arrays. */
typedef struct nb_batch nb_batch;
int nb_batch_create(nb_batch **batch, int nprob, const int *nelx, const int *nely,
                    const int *nelz, const int *lx1);
int nb_batch_destroy(nb_batch *batch);
/* total points, total elements, number of distinct lx1 */
int nb_batch_info(const nb_batch *batch, long *npts, int *nelt, int *nlx);
int nb_batch_problem(const nb_batch *batch, int prob, long *pt_offset, long *npts,
                     int *lx1);
/* device pointers of the concatenated x, f, c (n each) and g (6n) */
int nb_batch_arrays(nb_batch *batch, double **x, double **f, double **g, double **c);
/* g = setup_g form, c = inverse multiplicity, f of problem p = the
 * nb_rhs_uniform right-hand side with seed + p */
int nb_batch_setup(nb_batch *batch, uint64_t seed);
/* Autotuner: times every instantiated shape (elements per block, D in
 * registers or shared memory) of the FP32 inner and FP64 defect element
 * operators on the batch's elements of each lx1, reps launches each, and
 * keeps the fastest.  Overwrites x.  The FP64 defect's shapes: epb64 = -1
 * the fixed-point form on the integer pipes (the default before tuning),
 * 0 the even-odd form on the FP64 pipe, > 0 elements per block. */
int nb_batch_tune(nb_batch *batch, int reps);
int nb_batch_get_tuning(const nb_batch *batch, int lx1, int *epb32, int *rd32, int *epb64,
                        float *ms32, float *ms64);
int nb_batch_set_tuning(nb_batch *batch, int lx1, int epb32, int rd32, int epb64);
/* Enqueues the solve of every problem to |r|_C / |f|_C <= tol (cycles of
 * inner_iters FP32 CG iterations, at most max_outer cycles) as one graph
 * launch on the library stream; x starts at 0. */
int nb_batch_solve(nb_batch *batch, double tol, int inner_iters, int max_outer);
/* Diagnostic: the same solve, same kernels and same results, launched one
 * cycle at a time (each cycle a graph with an event after every launch, the
 * loop condition read on the host between cycles), and synchronous.  ms[7]
 * gets each phase's device time summed over the solve: 0 initial norms,
 * 1 cycle start (scale r into the FP32 right-hand side), 2 inner element
 * operator, 3 inner gather-scatter and p'Ap, 4 inner x/r/p update, 5 FP64
 * defect element operator, 6 defect gather-scatter and residual norm;
 * cycles gets the cycles run.  The loop-condition kernel of the graph solve
 * (one block per cycle) is not part of it. */
int nb_batch_time_phases(nb_batch *batch, double tol, int inner_iters, int max_outer,
                         double *ms, int *cycles);
/* Inner stopping of later solves: 0 (default) every cycle runs inner_iters
 * FP32 iterations; itol in (0, 1) ends each problem's inner CG once its
 * r'Cr fell by itol^2 (its residual by itol), at most inner_iters. */
int nb_batch_set_inner_tol(nb_batch *batch, double itol);
/* per problem: cycles, inner iterations, final |r|_C / |f|_C (synchronises) */
int nb_batch_result(const nb_batch *batch, int prob, int *outer, int *inner, double *relres);
/* cycles the last solve's loop ran */
int nb_batch_cycles(const nb_batch *batch, int *cycles);
/* asynchronous copies of the whole concatenated f in / x out (pinned host
 * buffers of nb_batch_info's npts doubles) */
int nb_batch_rhs_in(nb_batch *batch, const double *f_host);
int nb_batch_x_out(nb_batch *batch, double *x_host);

#ifdef __cplusplus
}
#endif
#endif

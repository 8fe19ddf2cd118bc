// nb_solver.h -- device-resident operator and CG solver state.
#pragma once

#include <memory>
#include <vector>

#include "nb_internal.h"
#include "nb_kernels.cuh"

namespace nb {

// A mesh with its gather-scatter topology, the derivative matrix and the
// Dirichlet mask, all resident on the device.
struct Operator {
  int nelx = 0, nely = 0, nelz = 0, nelt = 0, lx = 0;
  long n = 0;
  std::vector<int> lglel;          // global element numbers (1-based)
  std::vector<double> D;           // dxm1, column-major
  double *dD = nullptr;
  float *fD = nullptr;
  // even-odd split of D (E, O of D and of D^T, 4*(lx/2)^2), kept on the
  // host: each launch passes them as a kernel parameter.  Valid when lx is
  // even and D is anti-centrosymmetric to rounding
  std::vector<double> EO;
  bool eo_ok = false;
  // the same tables in fixed point for the FP64 operator on the integer
  // pipes (nb_ax_fx.cuh): balanced halves, fx_fc fractional bits
  std::vector<int> FXhi, FXlo;
  int fx_fc = 0;
  bool fx_ok = false;
  // the metric of the solve in progress in fixed point (metric_fx_prepare):
  // balanced halves per value, one exponent per element, converted from
  // gfx_src
  mutable int2 *gfx = nullptr;
  mutable int *gexp = nullptr;
  mutable const double *gfx_src = nullptr;
  mutable long gfx_cap = 0;
  int order = 2;                   // 0 reference left-to-right sums, 1 even-odd
                                   // (FP64 and FP32 operators alike), 2 (default)
                                   // the FP64 operator in fixed point where the
                                   // even-odd tables exist (FP32: even-odd)
  GsHost gsh_host;                 // jl maps of the dssum handle
  GsDevice gs;                     // device form
  // mask state (maskit, cg.f:214-258)
  int mask_mode = 1;               // 0 reference list semantics, 1 full
  bool mask_built = false;         // reference mode: list built
  std::vector<int> mask_list;      // masked local indices (deduplicated)
  int *d_mask_list = nullptr;
  int n_mask = 0;
  std::vector<unsigned char> face;  // per-element domain faces (get_face)
  unsigned char *d_face = nullptr;
  // fused gather-scatter over element boundary points
  bool fused_ok = false;
  int nbg = 0;
  long nbnd = 0;                    // members over all boundary groups
  std::vector<int> bnd_off_h;
  std::vector<unsigned> bnd_idx_h;  // without mask flags
  int *bnd_off = nullptr;
  unsigned *bnd_idx = nullptr;      // with mask flags in bit 31
  cudaStream_t stream = nullptr;
  bool brick = false;               // box in the brick element order (lglel(e) = e)

  ~Operator();
};

// Work space of one CG solve (reduction partials, scalars, history).
struct CgWork {
  double *partial_ax = nullptr, *partial_gs = nullptr, *partial_up = nullptr,
         *partial_dot = nullptr;
  unsigned *counters = nullptr;  // [0] gs_fin, [1] update, [2] glsc3
  CgScalars *sc = nullptr;
  double *hist = nullptr;
  int hist_len = 0;
  double *dot_out = nullptr;
  int grid_up = 0, grid_gs = 0, cap_ax = 0;
  // vector scratch of the solvers to a tolerance (kept between calls, so a
  // repeated solve allocates nothing)
  unsigned char *scratch = nullptr;
  size_t scratch_bytes = 0;
  // the FP32 metric of the solve in progress has one block for all
  // elements (set by the mixed solver around its inner CG)
  int g32_uniform = 0;
  // the preconditioner's FP32 input holds float(r) of the current r
  bool r32_ready = false;
  // an FP32 solve in progress takes its element products on the tensor
  // cores (unfused iteration; set by the mixed solver around its inner CG)
  bool tc_inner = false;
  // an FP32 solve in progress whose c verified as the closed-form
  // multiplicity (c_closed_form): each element's face bits; the fused
  // iteration then forms c instead of reading it (same values)
  const unsigned char *c32_face = nullptr;
  // the FP64 CG's second direction buffer (paired x update)
  double *palt = nullptr;
  long palt_n = 0;
  ~CgWork();
  int ensure(const Operator &op, int niter);
  int ensure_scratch(size_t bytes);
  int ensure_palt(long n);
};

// Builds the operator for a box of nelx*nely*nelz elements with lx points
// per direction on the reference's brick decomposition (init_mesh,
// driver.f:117-194) and numbering (set_vert_box, prox_dssum.f:42-73).
int operator_box(Operator *op, int nelx, int nely, int nelz, int lx,
                 int mask_mode, cudaStream_t s);
// Operator from a caller's mesh description and existing jl maps.
int operator_from(Operator *op, int nelx, int nely, int nelz, int nelt,
                  int lx, const int *lglel, const double *dxm1,
                  const GsHost &maps, int mask_mode, cudaStream_t s);
// E, O of D and of D^T (4*(lx/2)^2 values) when lx is even and D is
// anti-centrosymmetric to rounding (the even-odd contraction form).
bool even_odd_tables(const std::vector<double> &D, int lx, std::vector<double> &eo);
// The even-odd tables in fixed point (nb_ax_fx.cu): balanced 32-bit halves of
// round(C 2^fc), |round(C 2^fc)| <= 2^59, from D's exact values.
bool fx_tables(const std::vector<double> &D, int lx, std::vector<int> &hi,
               std::vector<int> &lo, int *fc);
// The metric g in the fixed-point operator's form, converted when g is not
// the array last converted (one pass over g); metric_fx_invalidate forgets
// the conversion (every solve and every standalone apply starts with it, so
// a caller may change g's contents between calls).
int metric_fx_prepare(const Operator &op, const double *g, cudaStream_t s);
void metric_fx_invalidate(const Operator &op);
// The mesh-independent part of an operator: sizes, element numbers, D and
// its even-odd tables, the domain faces of every element.
int operator_base(Operator *op, int nelx, int nely, int nelz, int nelt, int lx,
                  const int *lglel, const double *dxm1, int mask_mode, cudaStream_t s);
// The gather-scatter groups and the fused boundary groups of a brick-ordered
// box, built on the device without a sort (nb_topo.cu).  Mask mode 1 also
// gets the full Dirichlet mask list and the members' mask flags; mode 0
// starts unmasked (maskit builds its list on first use).  The host jl maps
// stay empty: every later use (gather-scatter, multigrid set-up) runs on
// the device maps.
int box_topology_device(Operator *op, cudaStream_t s);
// Whether glo_num (n points) is set_vert_box's numbering of a box in the
// brick element order (lglel(e) = e): the sizes are read off the first
// points, then every point is checked on the device.  On success *lx,
// *nelx, *nely, *nelz hold the box.
int box_numbering(const int64_t *glo_num, long n, bool *is_box, int *lx, int *nelx,
                  int *nely, int *nelz, cudaStream_t s);
// The gather-scatter CSR alone for lx points per element direction on the
// same brick (the multigrid levels' regular and extended numberings).
int box_gs_device(int lx, int nelx, int nely, int nelz, GsDevice *g, cudaStream_t s);
// Whether operator_box builds full-mask topologies on the device (default
// on); the host path (jl's sort-based construction) stays available.
bool setup_on_device();
void set_setup_on_device(bool on);
// Re-derives the device mask list and the fused-path mask flags.
int operator_set_mask(Operator *op, const std::vector<int> &list);
// Full Dirichlet mask of every element's domain faces (get_face per element).
std::vector<int> full_mask_list(const Operator &op);

// ------------------------------------------------------------- kernels --
template <typename T>
int launch_ax(const Operator &op, int mode, AxArgs<T> a, cudaStream_t s);
template <>
int launch_ax<double>(const Operator &op, int mode, AxArgs<double> a, cudaStream_t s);
template <>
int launch_ax<float>(const Operator &op, int mode, AxArgs<float> a, cudaStream_t s);
// The fixed-point FP64 operator in MODE 2 on op's tables (op.lx, FXhi,
// FXlo, fx_fc) for a.nelt elements; a.gfx / a.gexp set by the caller.
int launch_ax_fx_m2(const Operator &op, AxArgs<double> a, cudaStream_t s);
template <typename T>
int vec_glsc3(const T *a, const T *b, const T *m, long n, CgWork &wk,
              double *out, CgScalars *sc, int mode, int iter, cudaStream_t s,
              const float *mf = nullptr, T *mout = nullptr);
template <typename T>
int vec_add2s1(T *a, const T *b, const double *c1_dev, double c1, long n,
               cudaStream_t s);
template <typename T>
int vec_add2s2(T *a, const T *b, double c1, long n, cudaStream_t s);
template <typename T>
int vec_mask(T *w, const int *list, int nlist, cudaStream_t s);
template <typename T>
int vec_copy(T *a, const T *b, long n, cudaStream_t s);
template <typename T, typename S>
int vec_convert(T *a, const S *b, long n, cudaStream_t s);

// w = mask(QQ^T A_L u + 0.1 u)  (ax, cg.f:96-125), unfused path.
template <typename T>
int apply_ax(const Operator &op, T *w, const T *u, const T *g, cudaStream_t s);
// the same in FP32 with the element products on the tensor cores (nb_ax_tc.cu)
int apply_ax_tc(const Operator &op, float *w, const float *u, const float *g, cudaStream_t s);

// CG of cg.f:2-84 on device data.  z may equal r (identity preconditioner).
// precond: nullptr for the identity (hsmg_dum.f), else z = M^-1 r.
struct Precond {
  virtual int apply(double *z, double *r, cudaStream_t s) = 0;
  // An FP32 preconditioner on an r that is already masked may take its
  // input as float(r) written by the CG update (r32_in, null when it cannot)
  // and leave its result in FP32 (z32_out) for the r.z product to convert:
  // apply_f32 runs it from that input.
  virtual float *r32_in() { return nullptr; }
  virtual int apply_f32(cudaStream_t) { return 1; }
  virtual const float *z32_out() { return nullptr; }
  virtual ~Precond() {}
};
int cg_device(Operator &op, CgWork &wk, double *x, const double *f,
              const double *g, const double *c, double *r, double *w,
              double *p, double *z, int niter, Precond *M, bool force_unfused,
              cudaStream_t s);
// The same iteration split in two: the set-up of cg.f:36-42, then
// iterations it0..it1 (identity preconditioner), scalars kept on the device.
int cg_begin(Operator &op, CgWork &wk, double *x, const double *f,
             const double *c, double *r, int niter, cudaStream_t s);
int cg_steps(Operator &op, CgWork &wk, double *x, const double *g,
             const double *c, double *r, double *w, double *p, int it0,
             int it1, cudaStream_t s);
// mixed solver's fused defect pass: x += scale*e (e may be null);
// r = f - A x; r'Cr into wk.sc->rtr (fused path only)
int residual_fused(Operator &op, CgWork &wk, double *x, const float *e,
                   double scale, const double *f, const double *g,
                   const double *c, double *r, double *w, cudaStream_t s);
// CUDA-event times of the three kernels of a fused CG iteration, in the
// solvers' form: with the paired x update (nb_set_paired_update) the
// average over pairs of iterations; FP32 with c in closed form where it
// verifies (nb_set_mixed_closed_multiplicity)
template <typename T>
int time_cg_kernels_t(Operator &op, CgWork &wk, T *x, const T *f, const T *g,
                      const T *c, T *r, T *w, T *p, int reps, double *ms3,
                      cudaStream_t s);
// the second and third kernels of a fused FP64 iteration, for timing
int launch_gs_fin(const Operator &op, CgWork &wk, double *w, const double *p,
                  const double *c, cudaStream_t s);
int launch_cg_update(const Operator &op, CgWork &wk, double *x, double *r,
                     const double *p, const double *w, const double *c,
                     int iter, cudaStream_t s);
// iterations it0..it1 with preconditioner M (z = M^-1 r), scalars on device
int cg_steps_pc(Operator &op, CgWork &wk, double *x, const double *g,
                const double *c, double *r, double *w, double *p, double *z,
                int it0, int it1, Precond *M, cudaStream_t s);
// nb_set_mixed_closed_multiplicity: the inner FP32 CGs (single mesh and
// batched) form c in closed form where it verifies (default true)
extern bool g_mixed_closed_c;
// nb_set_paired_update: the fused FP64 CG (cg_device) and the mixed
// solver's inner CG alternate two direction buffers and update x once per
// pair of iterations (default true)
extern bool g_paired_update;
// Whether the FP32 c is, bitwise at every point, 2^-m with m the number of
// the point's extreme local indices whose element face has a neighbour (a
// box mesh's inverse multiplicity): then *closed and cface[e] holds element
// e's face bits (bit 0/1 the faces i = 0 / lx-1, 2/3 for j, 4/5 for k).
// Even lx1 from 4 to 16 only.  flag: one device int; synchronises s.
int c_closed_form(const Operator &op, const float *c32, unsigned char *cface, int *flag,
                  bool *closed, cudaStream_t s);
// FP32 variant (inner solves of the mixed-precision path), x starts at 0.
// With p_alt (a second n-point direction buffer) the fused iterations
// alternate their directions between p and p_alt and update x once per two
// iterations (bitwise the same iterates, 8 fewer bytes a point per pair).
int cg_device_f32(Operator &op, CgWork &wk, float *x, const float *f,
                  const float *g, const float *c, float *r, float *w, float *p,
                  int niter, cudaStream_t s, float *p_alt = nullptr);

}  // namespace nb

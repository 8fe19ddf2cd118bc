// nb_mg.h -- hybrid Schwarz multigrid (hsmg.f) on the GPU.
#pragma once

#include <vector>

#include "nb_solver.h"

namespace nb {

struct MgLevel {
  int order = 0, nh = 0, nl = 0;  // polynomial order, points, extended points
  long n = 0, next = 0;           // nh^3*nelt, nl^3*nelt
  GsHost gs_host, gsx_host;       // regular and Schwarz (extended) numbering
  GsDevice gs, gsx;
  double *rstr_wt = nullptr;      // (nh,nh,2,3,nelt)   hsmg.f:201-249
  double *fast_s = nullptr;       // (nl*nl,2,3,nelt)   hsmg.f:285-378
  double *fast_d = nullptr;       // (nl^3,nelt)
  double *schwarz_wt = nullptr;   // (nh,nh,4,3,nelt)   hsmg.f:572-688
  int *mask = nullptr;            // masked points at this level
  int nmask = 0;
  double *jh = nullptr, *jht = nullptr;  // to the next finer level (nf x nc)
  double *e = nullptr, *r = nullptr;     // level vectors
  // FP32 copies for the FP32 smoother
  float *rstr_wt_f = nullptr, *fast_s_f = nullptr, *fast_d_f = nullptr,
        *schwarz_wt_f = nullptr, *jh_f = nullptr, *jht_f = nullptr, *e_f = nullptr,
        *r_f = nullptr;
};

struct Multigrid {
  const Operator *op = nullptr;
  int nlev = 0;
  MgLevel lv[8];                  // 1-based
  double *A = nullptr, *B = nullptr;  // extended work arrays (finest size)
  double *w = nullptr;            // interpolation result
  int precision = 64;             // 64, or 32: FP32 Schwarz smoother and transfers
  float *A_f = nullptr, *B_f = nullptr, *z_f = nullptr;
  // the levels below the finest run on a second stream beside the finest
  // level's smoother (the cycle is additive): their own extended work
  // arrays, the stream and the fork / join events
  double *A2 = nullptr, *B2 = nullptr;
  float *A2_f = nullptr, *B2_f = nullptr;
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // exact coarse solve (replacing the reference's copy + dssum): the
  // Galerkin operator R A P of the V-cycle's own transfer chain on the
  // unmasked vertices, probed with 27 colours, inverted densely
  bool coarse_exact = false;
  int nc = 0;                     // unmasked coarse vertices
  double *c_ainv = nullptr;       // nc x nc inverse, row-major (symmetric)
  int *c_gid = nullptr;           // level-1 local point -> coarse index or -1
  int *c_prim = nullptr;          // coarse index -> its first level-1 copy
  double *c_b = nullptr, *c_x = nullptr;
  ~Multigrid();
};

// h1mg_setup (hsmg.f:3-29).  orders == nullptr: the reference's level
// choice (h1mg_setup_mg_nx, hsmg.f:45-97; defined only for lx1 <= 10);
// otherwise nlev polynomial orders, coarsest first, the last = lx1-1.
int mg_setup(Multigrid *mg, const Operator &op, const int *orders, int nlev,
             cudaStream_t s, int precision = 64);
// Replaces the coarse "solve" (hsmg.f:945-957) by an exact solve of the
// Galerkin coarse operator for the metric g (FP64): probes R A P with 27
// colourings of the vertex grid, checks it reproduces R A P on a random
// vector and is symmetric, factors it (banded Cholesky) and keeps the dense
// inverse.  Box meshes in brick order, mask_mode 1, at most
// kMaxCoarse unknowns.
constexpr int kMaxCoarse = 16384;
int mg_setup_coarse(Multigrid *mg, const double *g, cudaStream_t s);
// the fixed-size FDM and transfer kernels (default) or the general ones only
void mg_set_fixed_kernels(bool on);
// h1mg_solve (hsmg.f:960-1034): z = M^-1 rhs; masks rhs in place.
int mg_solve(Multigrid &mg, double *z, double *rhs, cudaStream_t s);
// The FP32 cycle alone (precision 32): from the finest level's r_f, which
// the caller filled with float(rhs) of a masked rhs, to z_f.
int mg_solve_f32(Multigrid &mg, cudaStream_t s);

}  // namespace nb

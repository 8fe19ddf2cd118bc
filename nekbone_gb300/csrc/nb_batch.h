// nb_batch.h -- many independent box-mesh Poisson problems of uneven element
// counts and orders, solved together: one FP64 defect-correction loop around
// FP32 inner CG (the mixed solver of one mesh) for every problem at once,
// captured as one CUDA graph whose outer loop is a device-side conditional
// WHILE node.  The reference solves one mesh per process (driver.f:42-59);
// batching is new.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "nb_internal.h"
#include "nb_kernels.cuh"

namespace nb {

// Per-problem scalars, device resident.  The inner set (rtz1 .. rtr) is the
// FP32 CG of cg.f:48-75 with z = r; the outer set drives the defect loop.
struct BatchScalars {
  double rtz1, rtz2, beta, pap, alpha, rtr;  // inner CG
  double rn0, rn;                            // |f|_C and current |r|_C (FP64)
  double irtr0;                              // the cycle's first inner r'Cr
  double alpha_prev;                         // alpha of a deferred x update
  int active;                                // 1 while |r|/|f| > tol
  int outer, inner;                          // cycles and inner iterations
  int iactive;                               // 1 while the cycle's inner CG runs
  int pend;                                  // the inner CG stopped with its
                                             //   last x update deferred
};

// Per-problem index ranges into the concatenated batch arrays.
struct BatchProb {
  long pt0, n;      // points
  int el0, nelt;    // elements (global element index)
  int gc0, ngc;     // boundary-group chunks
  int pc0, npc;     // point chunks
  int lx;           // points per direction
  int ext0;         // its lx1's extreme-index table in the batch's ext4
};

// Launch shape of the batched element operator for one lx1.
struct BatchTune {
  int epb32 = 1;    // elements per block, FP32 inner operator
  int rd32 = 1;     // 1: D in registers + vector shared loads; 0: padded shared D;
                    // 2: even-odd, one 1-D line per thread (epb 1)
  int epb64 = 1;    // elements per block, FP64 defect operator (0: even-odd form)
  float ms32 = 0.f, ms64 = 0.f;  // measured time of the chosen shapes
};

// Arguments of the batched element operator (one lx1 group).
//   MODE 1 (FP32 inner CG): p = z + beta_p p (p = z at the first iteration);
//     w_L = A_L p; interior points finished (w = w_L + 0.1 p), element
//     partial of pap.
//   MODE 2 (FP64 defect): x += rn_p e; w_L = A_L x; interior points get
//     r = f - (w_L + 0.1 x) and the element partial of r'Cr.
template <typename T>
struct BaxArgs {
  T *w;
  const T *u;          // MODE 1: z
  T *p;                // MODE 1: search direction; MODE 2: x
  const T *pold;       // MODE 1: the old direction, read from here (another
                       //   buffer than p when the directions alternate; the
                       //   launcher sets it to p when null)
  const T *g, *c, *D;
  const T *f;          // MODE 2
  T *r;                // MODE 2
  const float *e;      // MODE 2: FP32 correction
  const double *eo_h;  // even-odd tables of D on the host (forms with epb 0 /
                       // rd 2): the launcher passes them as a kernel parameter
  const int *el_prob;  // element -> problem
  const BatchScalars *sc;
  double *partial;     // per element
  long pt0;            // first point of this lx1 group
  int el0, nel;        // element range of this lx1 group
  int first;           // MODE 1: first inner iteration
  unsigned *err;       // device error word (bounded waits on the metric copy)
  int wait_test;       // timeout self-test of that wait (block_copy_begin)
  int c_unit_interior;  // MODE 1: c verified as the inverse multiplicity, so 1
                        //   at element-interior points: not read there
};

// The batched element operator for one lx1 (T float: MODE 1, T double:
// MODE 2) with the given shape, one instantiation per supported lx1 (4, 6,
// 8, 10, 12).  Returns NB_ERR_UNSUPPORTED for a shape not instantiated.
template <int LX>
int batch_ax_f32_lx(int epb, int rd, const BaxArgs<float> &a, cudaStream_t s);
template <int LX>
int batch_ax_f64_lx(int epb, const BaxArgs<double> &a, cudaStream_t s);
// The FP64 defect operator's shape value for the fixed-point form (even
// lx1): x += |r| e by a streaming kernel, then the fixed-point element
// operator (nb_ax_fx.cuh) on the group's elements.
constexpr int kFxShape = -1;
// instantiated shapes for lx1 = lx: (elements per block, register D) for the
// FP32 operator, elements per block for the FP64 one (0: the even-odd form,
// kFxShape: fixed point)
std::vector<std::pair<int, int>> batch_shapes_f32(int lx);
std::vector<int> batch_shapes_f64(int lx);

}  // namespace nb

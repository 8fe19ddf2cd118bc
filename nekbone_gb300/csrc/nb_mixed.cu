// nb_mixed.cu -- device set-up helpers, FP64 CG to a tolerance, and the
// mixed-precision solver: FP32 inner CG (ax, gather-scatter and vector
// updates in FP32) inside an FP64 defect-correction loop.  The reference has
// no counterpart for these solvers (its cg runs a fixed niter, cg.f:48-75);
// they reuse the same operator, numbering, mask and norm
// sqrt(r'Cr) (cg.f:42,66-69).
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "../../include/nekbone_gb300.h"
#include "nb_solver.h"

namespace nb {

namespace {

int grid_for(long n) {
  return int(std::max(1L, std::min<long>(152L * 8, (n + 255) / 256)));
}

// setup_g (prox_setup.f:27-52) from the GLL weights
__global__ void k_setup_g(double *g, const double *wgt, int lx, long n) {
  const long l3 = long(lx) * lx * lx;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x) {
    const int r = int(q % l3);
    const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
    const double v = wgt[i] * wgt[j] * wgt[k];
    double *gp = g + 6 * q;
    gp[0] = v;
    gp[1] = 0.;
    gp[2] = 0.;
    gp[3] = v;
    gp[4] = 0.;
    gp[5] = v;
  }
}

// box global id of local point q (set_vert_box, prox_dssum.f:42-73) for the
// brick order lglel(e) = e
__global__ void k_rhs_uniform(double *f, int lx, int nelx, int nely, long n,
                              uint64_t seed) {
  const long l3 = long(lx) * lx * lx;
  const int nn = lx - 1;
  const long ax = long(nn) * nelx + 1, ay = long(nn) * nely + 1;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x) {
    const long e = q / l3;
    const int r = int(q % l3);
    const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
    const long ex = e % nelx, ey = (e / nelx) % nely, ez = e / (long(nelx) * nely);
    const long id = 1 + (nn * ex + i) + (nn * ey + j) * ax + (nn * ez + k) * ax * ay;
    f[q] = uniform_pm1(seed, uint64_t(id));
  }
}

__global__ void k_col2(double *a, const double *b, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = mul_rn(a[q], b[q]);
}

// r = f - w
__global__ void k_residual(double *r, const double *f, const double *w, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    r[q] = f[q] - w[q];
}

// x += scale * double(e)
__global__ void k_axpy_f32(double *x, const float *e, double scale, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    x[q] = fma_rn(scale, double(e[q]), x[q]);
}

// y = float(scale * r)
__global__ void k_scale_f32(float *y, const double *r, double scale, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    y[q] = float(r[q] * scale);
}

}  // namespace

int dev_setup_g(const Operator &op, double *g, cudaStream_t s) {
  const int lx = op.lx;
  std::vector<double> a(lx * lx), b(lx), c(lx * lx), d(lx * lx), z(lx);
  semhat(a.data(), b.data(), c.data(), d.data(), z.data(), lx - 1);
  double *dw = nullptr;
  NB_CUDA(cudaMalloc(&dw, lx * sizeof(double)));
  NB_CUDA(cudaMemcpy(dw, b.data(), lx * sizeof(double), cudaMemcpyHostToDevice));
  k_setup_g<<<grid_for(op.n), 256, 0, s>>>(g, dw, lx, op.n);
  NB_CUDA(cudaGetLastError());
  NB_CUDA(cudaStreamSynchronize(s));
  cudaFree(dw);
  return NB_OK;
}

// f = uniform[-1,1) per global point, dssum, times c, masked (the set_f
// sequence of driver.f:88-101 with a seeded, layout-independent source)
int dev_rhs_uniform(const Operator &op, double *f, const double *c,
                    uint64_t seed, cudaStream_t s) {
  k_rhs_uniform<<<grid_for(op.n), 256, 0, s>>>(f, op.lx, op.nelx, op.nely, op.n, seed);
  NB_CUDA(cudaGetLastError());
  NB_TRY(gs_exec(op.gs, f, 1, 1, 0, s));
  k_col2<<<grid_for(op.n), 256, 0, s>>>(f, c, op.n);
  NB_CUDA(cudaGetLastError());
  NB_TRY(vec_mask<double>(f, op.d_mask_list, op.n_mask, s));
  return NB_OK;
}

int dev_residual(const Operator &op, double *r, const double *f,
                 const double *w, long n, cudaStream_t s) {
  (void)op;
  k_residual<<<grid_for(n), 256, 0, s>>>(r, f, w, n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

int dev_axpy_f32(double *x, const float *e, double scale, long n, cudaStream_t s) {
  k_axpy_f32<<<grid_for(n), 256, 0, s>>>(x, e, scale, n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

int dev_scale_to_f32(float *y, const double *r, double scale, long n, cudaStream_t s) {
  k_scale_f32<<<grid_for(n), 256, 0, s>>>(y, r, scale, n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

cudaStream_t lib_stream();

}  // namespace nb

using namespace nb;

extern "C" {

// Declared here, defined in nb_abi.cpp: access to a mesh's operator/workspace.
int nb_mesh_parts(nb_mesh *mesh, void **op, void **wk);

int nb_cg_tol(nb_mesh *mesh, double *x, const double *f, const double *g,
              const double *c, double tol, int max_iter, int check_every,
              int *iters, double *relres) {
  clear_status();
  void *pop = nullptr, *pwk = nullptr;
  NB_TRY(nb_mesh_parts(mesh, &pop, &pwk));
  Operator &op = *static_cast<Operator *>(pop);
  CgWork &wk = *static_cast<CgWork *>(pwk);
  cudaStream_t s = lib_stream();
  const long n = op.n;
  if (check_every < 1) check_every = 1;
  NB_TRY(wk.ensure_scratch(size_t(3) * n * 8));
  double *r = reinterpret_cast<double *>(wk.scratch);
  double *w = r + n, *p = w + n;
  int done = 0;
  double rn0 = 0, rn = 0;
  // run CG in chunks: cg_device always starts from x=0, so iterate one long
  // solve with the device scalars and poll rnorm every check_every steps.
  int st = cg_begin(op, wk, x, f, c, r, max_iter, s);
  if (!st) {
    NB_CUDA(cudaMemcpyAsync(&rn0, &wk.sc->rnorm, 8, cudaMemcpyDeviceToHost, s));
    NB_CUDA(cudaStreamSynchronize(s));
    rn = rn0;
    while (done < max_iter && !st) {
      const int k = std::min(check_every, max_iter - done);
      st = cg_steps(op, wk, x, g, c, r, w, p, done + 1, done + k, s);
      done += k;
      NB_CUDA(cudaMemcpyAsync(&rn, &wk.sc->rnorm, 8, cudaMemcpyDeviceToHost, s));
      NB_CUDA(cudaStreamSynchronize(s));
      if (rn0 > 0 && rn / rn0 <= tol) break;
    }
  }
  if (st) return st;
  NB_TRY(device_error_check(s));
  if (iters) *iters = done;
  if (relres) *relres = rn0 > 0 ? rn / rn0 : 0.0;
  return NB_OK;
}

}  // extern "C"

namespace nb {
namespace {
// *same = 0 if any element's metric block (blk values) differs bitwise from
// element 0's: x indexes the block, y strides over elements 1..nelt-1
__global__ void k_metric_uniform(const unsigned *g, long blk, long nelt, int *same) {
  const long q = long(blockIdx.x) * blockDim.x + threadIdx.x;
  bool ok = true;
  if (q < blk) {
    const unsigned v = g[q];
    for (long e = 1 + blockIdx.y; e < nelt; e += gridDim.y) ok &= g[e * blk + q] == v;
  }
  if (!__syncthreads_and(ok) && threadIdx.x == 0) atomicExch(same, 0);
}
}  // namespace

// Whether every element of the FP32 metric g32 repeats element 0's block
// (a box of equal affine elements: the reference's own setup_g).  Then the
// element operator reads one cache-resident block instead of 24 B per point,
// with the same values, so the same results.
bool g_shared_metric = true;
void set_shared_metric(bool on) { g_shared_metric = on; }
// the inner CG's element products on the tensor cores (k_ax_tc: FP16 hi+lo
// split operands, FP32 accumulation) instead of the fused CUDA-core pass
bool g_mixed_tc = false;
// x updated once per two iterations from two direction buffers (the FP64
// CG, the mixed solver's inner CG and the batched solve's inner CG;
// bitwise the same iterates)
bool g_paired_update = true;
// the inner CGs (this solver's and the batched solve's) form c in closed
// form where c verifies as a box mesh's inverse multiplicity (the same
// values)
bool g_mixed_closed_c = true;

// flag: one device int of scratch
int metric_uniform(const float *g32, long nelt, int lx, int *flag, int *uniform,
                   cudaStream_t s) {
  const long blk = 6L * lx * lx * lx;
  const int one = 1;
  int h = 0;
  *uniform = 0;
  if (!g_shared_metric) return NB_OK;
  NB_CUDA(cudaMemcpyAsync(flag, &one, sizeof(int), cudaMemcpyHostToDevice, s));
  if (nelt > 1) {
    const dim3 grid(unsigned((blk + 255) / 256), unsigned(std::min<long>(nelt - 1, 1024)));
    k_metric_uniform<<<grid, 256, 0, s>>>(reinterpret_cast<const unsigned *>(g32), blk, nelt,
                                          flag);
    NB_CUDA(cudaGetLastError());
  }
  NB_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  NB_CUDA(cudaStreamSynchronize(s));
  *uniform = h;
  return NB_OK;
}
}  // namespace nb

extern "C" {

void nb_set_shared_metric(int on) { set_shared_metric(on != 0); }
void nb_set_mixed_tensor_cores(int on) { g_mixed_tc = on != 0; }
void nb_set_paired_update(int on) { g_paired_update = on != 0; }
void nb_set_mixed_closed_multiplicity(int on) { g_mixed_closed_c = on != 0; }

int nb_cg_mixed(nb_mesh *mesh, double *x, const double *f, const double *g,
                const double *c, double tol, int inner_iters, int max_outer,
                int *outer, int *inner_total, double *relres) {
  clear_status();
  void *pop = nullptr, *pwk = nullptr;
  NB_TRY(nb_mesh_parts(mesh, &pop, &pwk));
  Operator &op = *static_cast<Operator *>(pop);
  CgWork &wk = *static_cast<CgWork *>(pwk);
  cudaStream_t s = lib_stream();
  const long n = op.n;
  // reduction buffers (this may be the mesh's first solve), then scratch:
  // r, w (FP64); g32 (6n), c32, r32, e32, rr32, w32, p32, p32b (FP32); two
  // int flags; the elements' face bits (nelt bytes)
  int st = wk.ensure(op, std::max(inner_iters, 1));
  metric_fx_invalidate(op);
  const size_t flags_at = size_t(n) * (2 * 8 + 13 * 4);
  if (!st) st = wk.ensure_scratch(flags_at + 16 + size_t(op.nelt));
  if (st) return st;
  double *r = reinterpret_cast<double *>(wk.scratch);
  double *w = r + n;
  float *g32 = reinterpret_cast<float *>(w + n);
  float *c32 = g32 + 6 * n, *r32 = c32 + n, *e32 = r32 + n, *rr32 = e32 + n,
        *w32 = rr32 + n, *p32 = w32 + n, *p32b = p32 + n;
  int k = 0, inner = 0;
  double rn0 = 0.0, rn = 0.0;
  if (!st) st = vec_convert<float, double>(g32, g, 6 * n, s);
  if (!st) st = vec_convert<float, double>(c32, c, n, s);
  int uniform = 0;
  int *flag = reinterpret_cast<int *>(wk.scratch + flags_at);
  unsigned char *cface = wk.scratch + flags_at + 16;
  bool closed = false;
  if (!st) st = metric_uniform(g32, op.nelt, op.lx, flag, &uniform, s);
  if (!st && g_mixed_closed_c && op.fused_ok && !g_mixed_tc)
    st = c_closed_form(op, c32, cface, flag + 1, &closed, s);
  // x = 0, r = mask(f)
  if (!st && cudaMemsetAsync(x, 0, n * 8, s) != cudaSuccess) st = fail(NB_ERR_CUDA, "memset");
  if (!st) st = vec_copy<double>(r, f, n, s);
  if (!st) st = vec_mask<double>(r, op.d_mask_list, op.n_mask, s);
  const bool fused = op.fused_ok;
  if (!st) st = vec_glsc3<double>(r, c, r, n, wk, wk.dot_out + 3, nullptr, 0, 0, s);
  const double *rr_dev = wk.dot_out + 3;
  while (!st) {
    double rr = 0.0;
    if (cudaMemcpyAsync(&rr, rr_dev, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      st = fail(NB_ERR_CUDA, "nb_cg_mixed: reading the residual norm");
      break;
    }
    rn = std::sqrt(rr);
    if (k == 0) rn0 = rn;
    if (rn0 == 0.0 || rn / rn0 <= tol || k >= max_outer) break;
    // inner FP32 solve of A e = r / |r|
    st = dev_scale_to_f32(r32, r, 1.0 / rn, n, s);
    wk.g32_uniform = uniform;
    wk.tc_inner = g_mixed_tc;
    wk.c32_face = closed ? cface : nullptr;
    if (!st)
      st = cg_device_f32(op, wk, e32, r32, g32, c32, rr32, w32, p32, inner_iters, s,
                         g_paired_update ? p32b : nullptr);
    wk.g32_uniform = 0;
    wk.tc_inner = false;
    wk.c32_face = nullptr;
    // FP64 defect: x += |r| e; r = f - A x; r'Cr
    if (!st && fused) {
      st = residual_fused(op, wk, x, e32, rn, f, g, c, r, w, s);
      rr_dev = &wk.sc->rtr;
    } else if (!st) {
      st = dev_axpy_f32(x, e32, rn, n, s);
      if (!st) st = apply_ax<double>(op, w, x, g, s);
      if (!st) st = dev_residual(op, r, f, w, n, s);
      if (!st) st = vec_glsc3<double>(r, c, r, n, wk, wk.dot_out + 3, nullptr, 0, 0, s);
      rr_dev = wk.dot_out + 3;
    }
    inner += inner_iters;
    ++k;
  }
  if (st) return st;
  NB_TRY(device_error_check(s));
  if (outer) *outer = k;
  if (inner_total) *inner_total = inner;
  if (relres) *relres = rn0 > 0 ? rn / rn0 : 0.0;
  return NB_OK;
}

}  // extern "C"

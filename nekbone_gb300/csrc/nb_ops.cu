// nb_ops.cu -- single-call device kernels behind the reference's small
// entry points: mxm (mxm_wrapper.f:1-52), local_grad3 / local_grad3_t
// (cg.f:170-212) with caller-supplied D and Dt, and the glsc3 / add2s1 /
// add2s2 BLAS-1 routines (math.f:534-617) on device vectors.  Sums run left
// to right over the contracted index as mxfN does (mxm_std.f:255).
#include "nb_solver.h"

namespace nb {

namespace {

// c(i,j) = sum_k a(i,k) b(k,j); a(n1,n2), b(n2,n3), c(n1,n3) column-major
__global__ void k_mxm(const double *a, int n1, const double *b, int n2,
                      double *c, int n3) {
  const long q = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= long(n1) * n3) return;
  const int i = int(q % n1), j = int(q / n1);
  double s = mul_rn(a[i], b[long(j) * n2]);
  for (int k = 1; k < n2; ++k)
    s = fma_rn(a[i + long(k) * n1], b[k + long(j) * n2], s);
  c[q] = s;
}

// local_grad3, cg.f:170-187 (one thread per point)
__global__ void k_local_grad3(double *ur, double *us, double *ut,
                              const double *u, int m1, const double *D,
                              const double *Dt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int m2 = m1 * m1;
  if (q >= m2 * m1) return;
  const int i = q % m1, j = (q / m1) % m1, k = q / m2;
  double a = mul_rn(D[i], u[j * m1 + k * m2]);
  for (int m = 1; m < m1; ++m) a = fma_rn(D[i + m * m1], u[m + j * m1 + k * m2], a);
  ur[q] = a;
  double b = mul_rn(u[i + k * m2], Dt[j * m1]);
  for (int m = 1; m < m1; ++m) b = fma_rn(u[i + m * m1 + k * m2], Dt[m + j * m1], b);
  us[q] = b;
  double c = mul_rn(u[i + j * m1], Dt[k * m1]);
  for (int m = 1; m < m1; ++m) c = fma_rn(u[i + j * m1 + m * m2], Dt[m + k * m1], c);
  ut[q] = c;
}

// local_grad3_t, cg.f:189-212: u = Dt ur; w_k = us_k D; u += w; w = ut D; u += w
__global__ void k_local_grad3_t(double *u, const double *ur, const double *us,
                                const double *ut, int m1, const double *D,
                                const double *Dt, double *w) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int m2 = m1 * m1;
  if (q >= m2 * m1) return;
  const int i = q % m1, j = (q / m1) % m1, k = q / m2;
  double a = mul_rn(Dt[i], ur[j * m1 + k * m2]);
  for (int m = 1; m < m1; ++m) a = fma_rn(Dt[i + m * m1], ur[m + j * m1 + k * m2], a);
  double b = mul_rn(us[i + k * m2], D[j * m1]);
  for (int m = 1; m < m1; ++m) b = fma_rn(us[i + m * m1 + k * m2], D[m + j * m1], b);
  double c = mul_rn(ut[i + j * m1], D[k * m1]);
  for (int m = 1; m < m1; ++m) c = fma_rn(ut[i + j * m1 + m * m2], D[m + k * m1], c);
  u[q] = add_rn(add_rn(a, b), c);
  w[q] = c;
}

}  // namespace

int dev_mxm(const double *a, int n1, const double *b, int n2, double *c,
            int n3, cudaStream_t s) {
  const long tot = long(n1) * n3;
  if (tot <= 0 || n2 <= 0) return NB_OK;
  k_mxm<<<int((tot + 127) / 128), 128, 0, s>>>(a, n1, b, n2, c, n3);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

int dev_local_grad3(double *ur, double *us, double *ut, const double *u,
                    int n, const double *D, const double *Dt, cudaStream_t s) {
  const int m1 = n + 1, tot = m1 * m1 * m1;
  k_local_grad3<<<(tot + 127) / 128, 128, 0, s>>>(ur, us, ut, u, m1, D, Dt);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

int dev_local_grad3_t(double *u, const double *ur, const double *us,
                      const double *ut, int n, const double *D,
                      const double *Dt, double *w, cudaStream_t s) {
  const int m1 = n + 1, tot = m1 * m1 * m1;
  k_local_grad3_t<<<(tot + 127) / 128, 128, 0, s>>>(u, ur, us, ut, m1, D, Dt, w);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

}  // namespace nb

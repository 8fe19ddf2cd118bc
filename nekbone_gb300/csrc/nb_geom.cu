// nb_geom.cu -- geometric factors of a deformed box mesh.
//
// The reference only builds undeformed elements (setup_g, prox_setup.f:27-52:
// g1=g4=g6=w_i w_j w_k, g2=g3=g5=0).  For the deformed workloads each
// element is the trilinear image of its 8 vertices, and every vertex of the
// 2x2x2-per-element box (element size h = 2, as in the reference's reference
// element) is displaced by a smooth seeded field
//   d(X) = amp * h * sum_{q<4} a_q sin(k_q . X + phi_q)
// so shared vertices move together and the mesh stays conforming.  The
// factors are those ax_e (cg.f:156-163) expects:
//   G = w_i w_j w_k |J| J^-1 J^-T = w adj(J) adj(J)^T / det J,
//   (g1..g6) = (G11, G12, G13, G22, G23, G33), J = dx/dr.
// Mode parameters come from splitmix64(seed) so any host can reproduce them.
#include <cmath>
#include <vector>

#include "nb_solver.h"

namespace nb {

namespace {

struct Modes {
  double a[4][3], k[4][3], phi[4];
};

uint64_t splitmix64(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double unit(uint64_t &s) { return double(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

// a_q in [-1,1)^3, k_q = 2 pi m_q / L with integer m_q in [1,3] per
// direction (L = the box extent), phi_q in [0, 2 pi)
Modes make_modes(uint64_t seed, int nelx, int nely, int nelz) {
  Modes M;
  uint64_t s = seed;
  const double L[3] = {2.0 * nelx, 2.0 * nely, 2.0 * nelz};
  const double twopi = 8.0 * std::atan(1.0);
  for (int q = 0; q < 4; ++q) {
    for (int d = 0; d < 3; ++d) M.a[q][d] = 2.0 * unit(s) - 1.0;
    for (int d = 0; d < 3; ++d) M.k[q][d] = twopi * double(1 + int(splitmix64(s) % 3)) / L[d];
    M.phi[q] = twopi * unit(s);
  }
  return M;
}

__global__ void k_setup_g_deformed(double *g, const double *z, const double *w,
                                   int lx, int nelx, int nely, long n, Modes M,
                                   double amp) {
  const long l3 = long(lx) * lx * lx;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x) {
    const long e = q / l3;
    const int rr = int(q % l3);
    const int i = rr % lx, j = (rr / lx) % lx, k = rr / (lx * lx);
    const int ex = int(e % nelx), ey = int((e / nelx) % nely), ez = int(e / (long(nelx) * nely));
    // the 8 displaced vertices
    double X[8][3];
    for (int v = 0; v < 8; ++v) {
      const double P[3] = {2.0 * (ex + (v & 1)), 2.0 * (ey + ((v >> 1) & 1)),
                           2.0 * (ez + ((v >> 2) & 1))};
      for (int d = 0; d < 3; ++d) {
        double dd = 0.0;
        for (int m = 0; m < 4; ++m)
          dd += M.a[m][d] *
                sin(M.k[m][0] * P[0] + M.k[m][1] * P[1] + M.k[m][2] * P[2] + M.phi[m]);
        X[v][d] = P[d] + amp * 2.0 * dd;
      }
    }
    const double r = z[i], s = z[j], t = z[k];
    double J[3][3] = {{0}};  // J[a][b] = dx_a / dr_b
    for (int v = 0; v < 8; ++v) {
      const double sr = (v & 1) ? 1.0 : -1.0, ss = ((v >> 1) & 1) ? 1.0 : -1.0,
                   st = ((v >> 2) & 1) ? 1.0 : -1.0;
      const double fr = 0.5 * (1 + sr * r), fs = 0.5 * (1 + ss * s), ft = 0.5 * (1 + st * t);
      const double dr = 0.5 * sr * fs * ft, ds = 0.5 * ss * fr * ft, dt = 0.5 * st * fr * fs;
      for (int a = 0; a < 3; ++a) {
        J[a][0] += dr * X[v][a];
        J[a][1] += ds * X[v][a];
        J[a][2] += dt * X[v][a];
      }
    }
    // adjugate: C = adj(J) = det(J) J^-1
    double C[3][3];
    C[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    C[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    C[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    C[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    C[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    C[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    C[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    C[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    C[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double det = J[0][0] * C[0][0] + J[0][1] * C[1][0] + J[0][2] * C[2][0];
    const double wq = w[i] * w[j] * w[k] / det;
    double G[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        G[a][b] = wq * (C[a][0] * C[b][0] + C[a][1] * C[b][1] + C[a][2] * C[b][2]);
    double *gp = g + 6 * q;
    gp[0] = G[0][0];
    gp[1] = G[0][1];
    gp[2] = G[0][2];
    gp[3] = G[1][1];
    gp[4] = G[1][2];
    gp[5] = G[2][2];
  }
}

}  // namespace

int dev_setup_g_deformed(const Operator &op, double *g, uint64_t seed, double amp,
                         cudaStream_t s) {
  const int lx = op.lx;
  std::vector<double> a(lx * lx), b(lx), c(lx * lx), d(lx * lx), z(lx);
  semhat(a.data(), b.data(), c.data(), d.data(), z.data(), lx - 1);
  double *dz = nullptr, *dw = nullptr;
  NB_CUDA(cudaMalloc(&dz, lx * sizeof(double)));
  NB_CUDA(cudaMalloc(&dw, lx * sizeof(double)));
  NB_CUDA(cudaMemcpy(dz, z.data(), lx * sizeof(double), cudaMemcpyHostToDevice));
  NB_CUDA(cudaMemcpy(dw, b.data(), lx * sizeof(double), cudaMemcpyHostToDevice));
  const Modes M = make_modes(seed, op.nelx, op.nely, op.nelz);
  const int grid = int(std::max(1L, std::min<long>(152L * 8, (op.n + 255) / 256)));
  k_setup_g_deformed<<<grid, 256, 0, s>>>(g, dz, dw, lx, op.nelx, op.nely, op.n, M, amp);
  NB_CUDA(cudaGetLastError());
  NB_CUDA(cudaStreamSynchronize(s));
  cudaFree(dz);
  cudaFree(dw);
  return NB_OK;
}

}  // namespace nb

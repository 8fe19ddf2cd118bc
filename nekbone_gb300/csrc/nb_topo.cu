// nb_topo.cu -- the gather-scatter topology of a box mesh, built on the
// device without a sort.
//
// For the reference's brick element order (lglel(e) = e, init_mesh,
// driver.f:179-190) and box numbering (set_vert_box, prox_dssum.f:42-73),
// the local copies of a global point are known in closed form: along each
// direction a point on an element face (i = 0 or lx1-1) is shared with the
// neighbouring element at the opposite face index.  Enumerating the
// neighbour options z-major, then y, then x, each in increasing element
// coordinate, lists the copies in increasing local index -- the member order
// of jl's local map (gs.c:88-113, 330-357: members by ascending local index,
// the first one the primary).  A point starts a group when it is its own
// first copy; groups therefore come out in ascending primary order, which is
// jl's group order, with an exclusive scan over the points.
//
// Three products, in one classify / scan / emit sweep:
//   * the gather-scatter CSR of every group of two or more copies (jl's map);
//   * the fused pass's boundary groups: every element-boundary point's group,
//     singletons included, members on a domain face flagged in bit 31;
//   * the full Dirichlet mask list (every element's domain-face points).
#include <algorithm>
#include <vector>

#include "nb_solver.h"

namespace nb {

namespace {

constexpr int kPts = 8;             // points per thread
constexpr int kThr = 256;
constexpr int kBlk = kPts * kThr;   // points per block

struct Box {
  int lx, nelx, nely, nelz;
  long n;
};

struct PointInfo {
  int m;          // number of copies
  int q[8];       // copies, ascending
  bool primary;   // q[0] is the point itself
  bool boundary;  // on an element face
  bool masked;    // on a domain face
};

__device__ __forceinline__ void classify(const Box &b, long q, PointInfo &pi) {
  const int lx = b.lx, nn = lx - 1;
  const long l3 = long(lx) * lx * lx;
  const long e = q / l3;
  const int r = int(q - e * l3);
  const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
  const int ex = int(e % b.nelx), ey = int((e / b.nelx) % b.nely),
            ez = int(e / (long(b.nelx) * b.nely));
  int xe[2], xi[2], ye[2], yi[2], ze[2], zi[2];
  int nx = 1, ny = 1, nz = 1;
  xe[0] = ex, xi[0] = i;
  if (i == 0 && ex > 0) { xe[0] = ex - 1; xi[0] = nn; xe[1] = ex; xi[1] = 0; nx = 2; }
  else if (i == nn && ex < b.nelx - 1) { xe[1] = ex + 1; xi[1] = 0; nx = 2; }
  ye[0] = ey, yi[0] = j;
  if (j == 0 && ey > 0) { ye[0] = ey - 1; yi[0] = nn; ye[1] = ey; yi[1] = 0; ny = 2; }
  else if (j == nn && ey < b.nely - 1) { ye[1] = ey + 1; yi[1] = 0; ny = 2; }
  ze[0] = ez, zi[0] = k;
  if (k == 0 && ez > 0) { ze[0] = ez - 1; zi[0] = nn; ze[1] = ez; zi[1] = 0; nz = 2; }
  else if (k == nn && ez < b.nelz - 1) { ze[1] = ez + 1; zi[1] = 0; nz = 2; }
  int m = 0;
  for (int c = 0; c < nz; ++c)
    for (int bb = 0; bb < ny; ++bb)
      for (int a = 0; a < nx; ++a) {
        const long ee = xe[a] + long(b.nelx) * (ye[bb] + long(b.nely) * ze[c]);
        pi.q[m++] = int(ee * l3 + xi[a] + lx * yi[bb] + lx * lx * zi[c]);
      }
  pi.m = m;
  pi.primary = pi.q[0] == int(q);
  pi.boundary = i == 0 || i == nn || j == 0 || j == nn || k == 0 || k == nn;
  pi.masked = (i == 0 && ex == 0) || (i == nn && ex == b.nelx - 1) || (j == 0 && ey == 0) ||
              (j == nn && ey == b.nely - 1) || (k == 0 && ez == 0) ||
              (k == nn && ez == b.nelz - 1);
}

// per point: [0] gs groups, [1] gs members, [2] boundary groups, [3] their
// members, [4] masked points
__device__ __forceinline__ void counts(const PointInfo &pi, int *c) {
  const bool g = pi.primary && pi.m >= 2;
  const bool bd = pi.primary && pi.boundary;
  c[0] = g ? 1 : 0;
  c[1] = g ? pi.m : 0;
  c[2] = bd ? 1 : 0;
  c[3] = bd ? pi.m : 0;
  c[4] = pi.masked ? 1 : 0;
}

// exclusive block scan of 5 counters held per thread; returns the block's
// prefix for this thread in pre[], block totals in tot[]
__device__ __forceinline__ void block_scan5(const int *v, int *pre, int *tot) {
  __shared__ int sh[5][kThr];
  const int t = threadIdx.x;
  for (int c = 0; c < 5; ++c) sh[c][t] = v[c];
  __syncthreads();
  // Hillis-Steele inclusive scan, 5 lanes at once
  for (int off = 1; off < kThr; off <<= 1) {
    int add[5];
    for (int c = 0; c < 5; ++c) add[c] = t >= off ? sh[c][t - off] : 0;
    __syncthreads();
    for (int c = 0; c < 5; ++c) sh[c][t] += add[c];
    __syncthreads();
  }
  for (int c = 0; c < 5; ++c) {
    pre[c] = sh[c][t] - v[c];
    tot[c] = sh[c][kThr - 1];
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThr) k_topo_count(Box b, int *blocksum) {
  const long q0 = long(blockIdx.x) * kBlk + long(threadIdx.x) * kPts;
  int v[5] = {0, 0, 0, 0, 0};
  for (int p = 0; p < kPts; ++p) {
    const long q = q0 + p;
    if (q >= b.n) break;
    PointInfo pi;
    classify(b, q, pi);
    int c[5];
    counts(pi, c);
    for (int k = 0; k < 5; ++k) v[k] += c[k];
  }
  int pre[5], tot[5];
  block_scan5(v, pre, tot);
  if (threadIdx.x == 0)
    for (int c = 0; c < 5; ++c) blocksum[c * gridDim.x + blockIdx.x] = tot[c];
}

// exclusive scan of the 5 block-sum arrays in place (one block); totals to
// total[0..4]
__global__ void __launch_bounds__(1024) k_topo_scan(int *blocksum, int nb, long *total) {
  __shared__ long carry[5];
  __shared__ long part[1024];
  const int t = threadIdx.x;
  for (int c = 0; c < 5; ++c) {
    if (t == 0) carry[c] = 0;
    __syncthreads();
    int *a = blocksum + long(c) * nb;
    for (int base = 0; base < nb; base += 1024) {
      const long v = base + t < nb ? a[base + t] : 0;
      part[t] = v;
      __syncthreads();
      for (int off = 1; off < 1024; off <<= 1) {
        const long add = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += add;
        __syncthreads();
      }
      if (base + t < nb) a[base + t] = int(carry[c] + part[t] - v);
      __syncthreads();
      if (t == 0) carry[c] += part[1023];
      __syncthreads();
    }
    if (t == 0) total[c] = carry[c];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThr)
    k_topo_emit(Box b, const int *blockpre, int *gs_off, int *gs_idx, int *bd_off,
                unsigned *bd_idx, int *mask, bool flags) {
  const long q0 = long(blockIdx.x) * kBlk + long(threadIdx.x) * kPts;
  int v[5] = {0, 0, 0, 0, 0};
  for (int p = 0; p < kPts; ++p) {
    const long q = q0 + p;
    if (q >= b.n) break;
    PointInfo pi;
    classify(b, q, pi);
    int c[5];
    counts(pi, c);
    for (int k = 0; k < 5; ++k) v[k] += c[k];
  }
  int pre[5], tot[5];
  block_scan5(v, pre, tot);
  int pos[5];
  for (int c = 0; c < 5; ++c) pos[c] = blockpre[c * gridDim.x + blockIdx.x] + pre[c];
  for (int p = 0; p < kPts; ++p) {
    const long q = q0 + p;
    if (q >= b.n) break;
    PointInfo pi;
    classify(b, q, pi);
    if (pi.primary && pi.m >= 2) {
      gs_off[pos[0]] = pos[1];
      for (int k = 0; k < pi.m; ++k) gs_idx[pos[1] + k] = pi.q[k];
      pos[0] += 1;
      pos[1] += pi.m;
    }
    if (bd_off && pi.primary && pi.boundary) {
      bd_off[pos[2]] = pos[3];
      for (int k = 0; k < pi.m; ++k)
        bd_idx[pos[3] + k] = unsigned(pi.q[k]) | (flags && pi.masked ? 0x80000000u : 0u);
      pos[2] += 1;
      pos[3] += pi.m;
    }
    if (mask && pi.masked) mask[pos[4]++] = int(q);
  }
}

bool g_setup_on_device = true;

}  // namespace

bool setup_on_device() { return g_setup_on_device; }
void set_setup_on_device(bool on) { g_setup_on_device = on; }

namespace {

// The sweep for lx points per element direction; bnd/mask outputs are
// produced only when op is given, the mask list and flags for mask mode 1.
int topology_sweep(const Box &b, GsDevice *g, Operator *op, cudaStream_t s) {
  if (b.n >= (1L << 31))
    return fail(NB_ERR_UNSUPPORTED, "device topology: n = %ld exceeds 2^31-1", b.n);
  const int nb = int((b.n + kBlk - 1) / kBlk);
  int *blocksum = nullptr;
  long *total = nullptr;
  NB_CUDA(cudaMalloc(&blocksum, size_t(5) * nb * sizeof(int)));
  NB_CUDA(cudaMalloc(&total, 5 * sizeof(long)));
  k_topo_count<<<nb, kThr, 0, s>>>(b, blocksum);
  k_topo_scan<<<1, 1024, 0, s>>>(blocksum, nb, total);
  long tot[5];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(tot, total, sizeof(tot), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaFree(blocksum);
    cudaFree(total);
    return fail(NB_ERR_CUDA, "device topology: %s", cudaGetErrorString(e));
  }
  *g = GsDevice();
  g->n = int(b.n);
  g->symmetric = true;
  g->ng = int(tot[0]);
  NB_CUDA(cudaMalloc(&g->off, (tot[0] + 1) * sizeof(int)));
  NB_CUDA(cudaMalloc(&g->idx, std::max(1L, tot[1]) * sizeof(int)));
  const bool full = op && op->mask_mode == 1;
  if (op) {
    op->nbg = int(tot[2]);
    op->nbnd = tot[3];
    op->n_mask = full ? int(tot[4]) : 0;
    NB_CUDA(cudaMalloc(&op->bnd_off, (tot[2] + 1) * sizeof(int)));
    NB_CUDA(cudaMalloc(&op->bnd_idx, std::max(1L, tot[3]) * sizeof(unsigned)));
    if (full) NB_CUDA(cudaMalloc(&op->d_mask_list, std::max(1L, tot[4]) * sizeof(int)));
  }
  k_topo_emit<<<nb, kThr, 0, s>>>(b, blocksum, g->off, g->idx, op ? op->bnd_off : nullptr,
                                  op ? op->bnd_idx : nullptr,
                                  full ? op->d_mask_list : nullptr, full);
  const int end_gs = int(tot[1]), end_bd = int(tot[3]);
  NB_CUDA(cudaMemcpyAsync(g->off + tot[0], &end_gs, sizeof(int), cudaMemcpyHostToDevice, s));
  if (op)
    NB_CUDA(cudaMemcpyAsync(op->bnd_off + tot[2], &end_bd, sizeof(int),
                            cudaMemcpyHostToDevice, s));
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(blocksum);
  cudaFree(total);
  if (e != cudaSuccess) return fail(NB_ERR_CUDA, "device topology: %s", cudaGetErrorString(e));
  return NB_OK;
}

}  // namespace

int box_topology_device(Operator *op, cudaStream_t s) {
  const Box b{op->lx, op->nelx, op->nely, op->nelz, op->n};
  NB_TRY(topology_sweep(b, &op->gs, op, s));
  op->fused_ok = true;
  op->mask_built = op->mask_mode == 1;
  op->brick = true;
  return NB_OK;
}

namespace {
// *bad = 1 where glo[q] differs from set_vert_box's value (prox_dssum.f:42-73)
// for the brick box b
__global__ void k_box_numbering(Box b, const long long *glo, int *bad) {
  const int lx = b.lx, nn = lx - 1;
  const long l3 = long(lx) * lx * lx;
  const long long ax = (long long)nn * b.nelx + 1, ay = (long long)nn * b.nely + 1;
  bool ok = true;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < b.n;
       q += long(gridDim.x) * blockDim.x) {
    const long e = q / l3;
    const int r = int(q - e * l3);
    const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
    const long long ex = e % b.nelx, ey = (e / b.nelx) % b.nely, ez = e / (long(b.nelx) * b.nely);
    const long long v = 1 + (nn * ex + i) + (nn * ey + j) * ax + (nn * ez + k) * ax * ay;
    ok &= glo[q] == v;
  }
  if (!__syncthreads_and(ok) && threadIdx.x == 0) atomicExch(bad, 1);
}
}  // namespace

int box_numbering(const int64_t *glo, long n, bool *is_box, int *lx_out, int *nelx_out,
                  int *nely_out, int *nelz_out, cudaStream_t s) {
  *is_box = false;
  // glo = q + 1 along element 0's first line; the line ends at q = lx
  long lx = 0;
  while (lx < n && lx < 64 && glo[lx] == lx + 1) ++lx;
  if (lx < 2 || lx >= 64) return NB_OK;
  const long l3 = lx * lx * lx;
  if (n < l3 || n % l3) return NB_OK;
  const long nn = lx - 1, nelt = n / l3;
  const long ax = glo[lx] - 1;                       // j = 1: 1 + ax
  if (ax < lx || (ax - 1) % nn) return NB_OK;
  const long nelx = (ax - 1) / nn;
  const long axy = glo[lx * lx] - 1;                 // k = 1: 1 + ax*ay
  if (axy < ax || axy % ax) return NB_OK;
  const long ay = axy / ax;
  if ((ay - 1) % nn) return NB_OK;
  const long nely = (ay - 1) / nn;
  if (nelx < 1 || nely < 1 || nelt % (nelx * nely)) return NB_OK;
  const long nelz = nelt / (nelx * nely);
  if (n >= (1L << 31)) return NB_OK;
  const Box b{int(lx), int(nelx), int(nely), int(nelz), n};
  long long *dglo = nullptr;
  int *bad = nullptr;
  NB_CUDA(cudaMalloc(&dglo, n * sizeof(long long)));
  cudaError_t e = cudaMalloc(&bad, sizeof(int));
  int hb = 1;
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dglo, glo, n * sizeof(long long), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_box_numbering<<<int(std::min<long>(152L * 8, (n + 255) / 256)), 256, 0, s>>>(b, dglo, bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dglo);
  if (bad) cudaFree(bad);
  if (e != cudaSuccess) return fail(NB_ERR_CUDA, "box_numbering: %s", cudaGetErrorString(e));
  if (!hb) {
    *is_box = true;
    *lx_out = int(lx), *nelx_out = int(nelx), *nely_out = int(nely), *nelz_out = int(nelz);
  }
  return NB_OK;
}

int box_gs_device(int lx, int nelx, int nely, int nelz, GsDevice *g, cudaStream_t s) {
  const Box b{lx, nelx, nely, nelz, long(nelx) * nely * nelz * lx * lx * lx};
  return topology_sweep(b, g, nullptr, s);
}

}  // namespace nb

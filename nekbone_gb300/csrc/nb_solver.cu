// nb_solver.cu -- device-resident operator set-up and the CG iteration.
//
// One CG iteration of cg.f:48-75 with the identity preconditioner is three
// kernels and no host round trip:
//   k_ax (MODE 1)   p = z + beta p; w_L = A_L p per element; interior points
//                   finished (w = w_L + 0.1 p); interior part of pap
//   k_gs_fin        jl-order sum over every group of element-boundary points,
//                   w = sum + 0.1 p, Dirichlet mask, boundary part of pap;
//                   last block forms pap and alpha
//   k_cg_update     x += alpha p, r -= alpha w, rtr; last block forms beta
// CG scalars stay on the device.  The unfused path (element product, jl
// gather-scatter, add2s2, maskit, glsc3 as separate kernels) covers meshes
// whose numbering shares element-interior points, and flagged handles.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "nb_solver.h"

namespace nb {

Operator::~Operator() {
  if (dD) cudaFree(dD);
  if (fD) cudaFree(fD);
  gs_release(&gs);
  if (d_mask_list) cudaFree(d_mask_list);
  if (d_face) cudaFree(d_face);
  if (bnd_off) cudaFree(bnd_off);
  if (bnd_idx) cudaFree(bnd_idx);
  if (gfx) cudaFree(gfx);
  if (gexp) cudaFree(gexp);
}

CgWork::~CgWork() {
  double *ps[] = {partial_ax, partial_gs, partial_up, partial_dot, hist, dot_out};
  for (double *p : ps)
    if (p) cudaFree(p);
  if (counters) cudaFree(counters);
  if (sc) cudaFree(sc);
  if (scratch) cudaFree(scratch);
  if (palt) cudaFree(palt);
}

int CgWork::ensure_palt(long n) {
  if (palt && palt_n >= n) return NB_OK;
  if (palt) cudaFree(palt);
  palt = nullptr;
  palt_n = 0;
  if (cudaMalloc(&palt, size_t(n) * sizeof(double)) != cudaSuccess)
    return fail(NB_ERR_CUDA, "CG direction buffer: out of device memory (%ld points)", n);
  palt_n = n;
  return NB_OK;
}

int CgWork::ensure_scratch(size_t bytes) {
  if (bytes <= scratch_bytes) return NB_OK;
  if (scratch) cudaFree(scratch);
  scratch = nullptr;
  scratch_bytes = 0;
  if (cudaMalloc(&scratch, bytes) != cudaSuccess)
    return fail(NB_ERR_CUDA, "solver scratch: out of device memory (%zu bytes)", bytes);
  scratch_bytes = bytes;
  return NB_OK;
}

static int sm_count() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 152;
  }
  return cached;
}

// Blocks per SM of the grid-stride boundary passes: exactly the resident
// ones (one wave).  At 32^3, lx1 = 12 (four resident blocks of 256) this
// took k_gs_fin from 0.440 to 0.404 ms (FP64) and 0.277 to 0.258 ms (FP32)
// against eight blocks per SM; five or six (a partial second wave) measured
// 0.52-0.60 ms.
static int gs_blocks_per_sm() {
  static int cached = 0;
  if (!cached) {
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_gs_fin<double>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_gs_fin<float>, 256, 0);
    cached = std::max(1, std::min(a, b));
  }
  return cached;
}

int CgWork::ensure(const Operator &op, int niter) {
  const int gu = int(std::max(1L, std::min<long>(sm_count() * 8L, (op.n + 255) / 256)));
  const int gg = int(std::max(
      1L, std::min<long>(long(sm_count()) * gs_blocks_per_sm(), (long(op.nbg) + 255) / 256)));
  if (!counters) {
    NB_CUDA(cudaMalloc(&counters, 8 * sizeof(unsigned)));
    NB_CUDA(cudaMemset(counters, 0, 8 * sizeof(unsigned)));
    NB_CUDA(cudaMalloc(&sc, sizeof(CgScalars)));
    NB_CUDA(cudaMemset(sc, 0, sizeof(CgScalars)));
    NB_CUDA(cudaMalloc(&dot_out, 8 * sizeof(double)));
  }
  const int need_ax = std::max(op.nelt, 1);
  if (need_ax > cap_ax || gu > grid_up || gg > grid_gs) {
    if (partial_ax) cudaFree(partial_ax);
    if (partial_gs) cudaFree(partial_gs);
    if (partial_up) cudaFree(partial_up);
    if (partial_dot) cudaFree(partial_dot);
    cap_ax = std::max(need_ax, cap_ax);
    grid_up = std::max(gu, grid_up);
    grid_gs = std::max(gg, grid_gs);
    NB_CUDA(cudaMalloc(&partial_ax, cap_ax * sizeof(double)));
    NB_CUDA(cudaMalloc(&partial_gs, grid_gs * sizeof(double)));
    NB_CUDA(cudaMalloc(&partial_up, grid_up * sizeof(double)));
    NB_CUDA(cudaMalloc(&partial_dot, grid_up * sizeof(double)));
  }
  grid_up = gu;
  grid_gs = gg;
  if (niter + 1 > hist_len) {
    if (hist) cudaFree(hist);
    hist_len = niter + 1;
    NB_CUDA(cudaMalloc(&hist, 5 * sizeof(double) * hist_len));
  }
  return NB_OK;
}

// ------------------------------------------------------------ set-up --
bool even_odd_tables(const std::vector<double> &D, int lx, std::vector<double> &eo) {
  if (lx % 2 != 0) return false;
  double dmax = 0.0, asym = 0.0;
  auto Dm = [&](int r, int c) { return D[r + c * lx]; };
  for (int r = 0; r < lx; ++r)
    for (int c = 0; c < lx; ++c) {
      dmax = std::max(dmax, std::fabs(Dm(r, c)));
      asym = std::max(asym, std::fabs(Dm(r, c) + Dm(lx - 1 - r, lx - 1 - c)));
    }
  if (asym > 1e-12 * dmax) return false;
  const int h = lx / 2;
  eo.assign(4 * h * h, 0.0);
  for (int a = 0; a < h; ++a)
    for (int m = 0; m < h; ++m) {
      eo[a * h + m] = (Dm(a, m) + Dm(a, lx - 1 - m)) / 2;
      eo[h * h + a * h + m] = (Dm(a, m) - Dm(a, lx - 1 - m)) / 2;
      eo[2 * h * h + a * h + m] = (Dm(m, a) + Dm(lx - 1 - m, a)) / 2;
      eo[3 * h * h + a * h + m] = (Dm(m, a) - Dm(lx - 1 - m, a)) / 2;
    }
  return true;
}

// Deals the lx^2 lines of one phase (line l starts in bank bank[l]) to the
// CTA's warps, 32 lanes each: a transportation problem from banks to warps,
// solved by max-flow with a per-(bank, warp) limit.  The limit starts at
// one line per bank in every warp and is raised one warp at a time until
// every line is placed.
static void deal_lines(int nt, const std::vector<int> &bank, unsigned char *map) {
  const int W = (nt + 31) / 32, N = 34 + W;  // 0 source, 1 sink, 2.. banks, 34.. warps
  std::vector<int> cnt(32, 0);
  for (int l = 0; l < nt; ++l) cnt[bank[l]]++;
  for (int extra = 0;; ++extra) {
    std::vector<int> cap(size_t(N) * N, 0);
    auto C = [&](int u, int v) -> int & { return cap[size_t(u) * N + v]; };
    for (int b = 0; b < 32; ++b) {
      C(0, 2 + b) = cnt[b];
      for (int w = 0; w < W; ++w) C(2 + b, 34 + w) = 1 + extra / W + (w < extra % W ? 1 : 0);
    }
    for (int w = 0; w < W; ++w) C(34 + w, 1) = std::min(32, nt - 32 * w);
    int flow = 0;
    for (;;) {
      std::vector<int> par(N, -1), q(1, 0);
      par[0] = 0;
      for (size_t h = 0; h < q.size() && par[1] < 0; ++h)
        for (int v = 0; v < N; ++v)
          if (par[v] < 0 && C(q[h], v) > 0) {
            par[v] = q[h];
            q.push_back(v);
          }
      if (par[1] < 0) break;
      int m = nt;
      for (int v = 1; v != 0; v = par[v]) m = std::min(m, C(par[v], v));
      for (int v = 1; v != 0; v = par[v]) {
        C(par[v], v) -= m;
        C(v, par[v]) += m;
      }
      flow += m;
    }
    if (flow != nt) continue;
    // the flow from bank b to warp w sits on the reverse edge
    std::vector<int> fill(W, 0);
    for (int l = 0; l < nt; ++l) {
      const int b = bank[l];
      for (int w = 0; w < W; ++w)
        if (C(34 + w, 2 + b) > 0) {
          C(34 + w, 2 + b)--;
          map[32 * w + fill[w]++] = (unsigned char)l;
          break;
        }
    }
    return;
  }
}

void eo_line_maps(int lx, int pl, unsigned char *rmap, unsigned char *smap) {
  const int nt = lx * lx;
  std::vector<int> br(nt), bs(nt);
  for (int k = 0; k < lx; ++k)
    for (int a = 0; a < lx; ++a) {
      br[a + lx * k] = (lx * a + pl * k) % 32;  // r-line (j = a, k): word j lx + k pl
      bs[a + lx * k] = (a + pl * k) % 32;       // s-line (i = a, k): word i + k pl
    }
  deal_lines(nt, br, rmap);
  deal_lines(nt, bs, smap);
}

static bool is_elem_boundary(long pt, int lx) {
  const long l3 = long(lx) * lx * lx;
  const int r = int(pt % l3);
  const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
  return i == 0 || i == lx - 1 || j == 0 || j == lx - 1 || k == 0 || k == lx - 1;
}

// Groups of element-boundary points for the fused pass: every gather-scatter
// group (all members must be element-boundary points) and every boundary
// point that belongs to no group, in order of the first member.
static void build_boundary_groups(Operator *op) {
  op->fused_ok = false;
  op->bnd_off_h.clear();
  op->bnd_idx_h.clear();
  if (!op->gs.symmetric) return;
  const long n = op->n;
  std::vector<int> grp(n, -1);  // >=0 group id at its primary, -2 member
  std::vector<int> goff;
  std::vector<int> gmem;
  {
    const uint32_t END = uint32_t(-1);
    const std::vector<uint32_t> &m = op->gsh_host.map[1];
    size_t q = 0;
    while (q < m.size() && m[q] != END) {
      const int g = int(goff.size());
      goff.push_back(int(gmem.size()));
      grp[m[q]] = g;
      gmem.push_back(int(m[q++]));
      while (m[q] != END) {
        grp[m[q]] = -2;
        gmem.push_back(int(m[q++]));
      }
      ++q;
    }
    goff.push_back(int(gmem.size()));
  }
  for (long pt = 0; pt < n; ++pt) {
    const bool b = is_elem_boundary(pt, op->lx);
    if (!b) {
      if (grp[pt] != -1) return;  // an interior point is shared
      continue;
    }
    if (grp[pt] == -2) continue;
    op->bnd_off_h.push_back(int(op->bnd_idx_h.size()));
    if (grp[pt] >= 0) {
      const int g = grp[pt];
      for (int q = goff[g]; q < goff[g + 1]; ++q) op->bnd_idx_h.push_back(unsigned(gmem[q]));
    } else {
      op->bnd_idx_h.push_back(unsigned(pt));
    }
  }
  op->bnd_off_h.push_back(int(op->bnd_idx_h.size()));
  op->nbg = int(op->bnd_off_h.size()) - 1;
  op->nbnd = long(op->bnd_idx_h.size());
  op->fused_ok = n < (1L << 31);
}

namespace {
// Mask flags of boundary-group members built on the device: bit 31 set
// exactly for the members in the sorted list (binary search).
__global__ void k_set_member_flags(unsigned *idx, long nm, const int *list, int nl) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < nm;
       q += long(gridDim.x) * blockDim.x) {
    const unsigned id = idx[q] & 0x7fffffffu;
    int lo = 0, hi = nl;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (unsigned(list[mid]) < id) lo = mid + 1;
      else hi = mid;
    }
    idx[q] = id | (lo < nl && unsigned(list[lo]) == id ? 0x80000000u : 0u);
  }
}
}  // namespace

std::vector<int> full_mask_list(const Operator &op) {
  std::vector<int> list;
  const int lx = op.lx;
  const long l3 = long(lx) * lx * lx;
  for (int e = 0; e < op.nelt; ++e) {
    const unsigned f = op.face[e];
    if (!f) continue;
    for (int k = 0; k < lx; ++k)
      for (int j = 0; j < lx; ++j)
        for (int i = 0; i < lx; ++i) {
          const bool m = ((f & 1u) && i == 0) || ((f & 2u) && i == lx - 1) ||
                         ((f & 4u) && j == 0) || ((f & 8u) && j == lx - 1) ||
                         ((f & 16u) && k == 0) || ((f & 32u) && k == lx - 1);
          if (m) list.push_back(int(l3 * e + i + lx * j + lx * lx * k));
        }
  }
  return list;
}

int operator_set_mask(Operator *op, const std::vector<int> &list_in) {
  std::vector<int> list = list_in;
  std::sort(list.begin(), list.end());
  list.erase(std::unique(list.begin(), list.end()), list.end());
  op->mask_list = list;
  if (op->d_mask_list) cudaFree(op->d_mask_list);
  op->d_mask_list = nullptr;
  op->n_mask = int(list.size());
  if (!list.empty()) {
    NB_CUDA(cudaMalloc(&op->d_mask_list, list.size() * sizeof(int)));
    NB_CUDA(cudaMemcpy(op->d_mask_list, list.data(), list.size() * sizeof(int),
                       cudaMemcpyHostToDevice));
  }
  if (op->nbg > 0 && op->bnd_idx_h.empty() && op->bnd_idx) {
    // groups built on the device (nb_topo.cu): flags set there
    for (int v : list)
      if (!is_elem_boundary(v, op->lx)) op->fused_ok = false;
    k_set_member_flags<<<int(std::max(1L, std::min<long>(152L * 8, (op->nbnd + 255) / 256))),
                         256, 0, op->stream>>>(op->bnd_idx, op->nbnd, op->d_mask_list,
                                               op->n_mask);
    NB_CUDA(cudaGetLastError());
    NB_CUDA(cudaStreamSynchronize(op->stream));
  } else if (op->nbg > 0 && !op->bnd_idx_h.empty()) {
    for (int v : list)
      if (!is_elem_boundary(v, op->lx)) op->fused_ok = false;
    std::vector<unsigned char> masked(op->n, 0);
    for (int v : list) masked[v] = 1;
    std::vector<unsigned> idx = op->bnd_idx_h;
    for (auto &v : idx)
      if (masked[v]) v |= 0x80000000u;
    if (!op->bnd_idx) {
      NB_CUDA(cudaMalloc(&op->bnd_idx, idx.size() * sizeof(unsigned)));
      NB_CUDA(cudaMalloc(&op->bnd_off, op->bnd_off_h.size() * sizeof(int)));
      NB_CUDA(cudaMemcpy(op->bnd_off, op->bnd_off_h.data(),
                         op->bnd_off_h.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    NB_CUDA(cudaMemcpy(op->bnd_idx, idx.data(), idx.size() * sizeof(unsigned),
                       cudaMemcpyHostToDevice));
  }
  return NB_OK;
}

int operator_base(Operator *op, int nelx, int nely, int nelz, int nelt, int lx,
                  const int *lglel, const double *dxm1, int mask_mode, cudaStream_t s) {
  if (lx < 2 || lx > kMaxLx)
    return fail(NB_ERR_UNSUPPORTED, "lx1=%d outside the supported range 2..%d", lx, kMaxLx);
  if (nelt <= 0) return fail(NB_ERR_ARG, "nelt=%d must be positive", nelt);
  op->nelx = nelx;
  op->nely = nely;
  op->nelz = nelz;
  op->nelt = nelt;
  op->lx = lx;
  op->n = long(nelt) * lx * lx * lx;
  op->stream = s;
  op->lglel.assign(lglel, lglel + nelt);
  op->D.assign(dxm1, dxm1 + lx * lx);
  op->mask_mode = mask_mode;
  NB_CUDA(cudaMalloc(&op->dD, lx * lx * sizeof(double)));
  NB_CUDA(cudaMalloc(&op->fD, lx * lx * sizeof(float)));
  std::vector<float> fDh(op->D.begin(), op->D.end());
  NB_CUDA(cudaMemcpy(op->dD, op->D.data(), lx * lx * sizeof(double), cudaMemcpyHostToDevice));
  NB_CUDA(cudaMemcpy(op->fD, fDh.data(), lx * lx * sizeof(float), cudaMemcpyHostToDevice));
  // even-odd tables when D(n-1-i,n-1-m) = -D(i,m) holds to rounding
  op->eo_ok = even_odd_tables(op->D, lx, op->EO);
  op->fx_ok = op->eo_ok && fx_tables(op->D, lx, op->FXhi, op->FXlo, &op->fx_fc);
  op->face.resize(nelt);
  for (int e = 0; e < nelt; ++e)
    op->face[e] = (unsigned char)face_bits(op->lglel[e], nelx, nely, nelz);
  NB_CUDA(cudaMalloc(&op->d_face, nelt));
  NB_CUDA(cudaMemcpy(op->d_face, op->face.data(), nelt, cudaMemcpyHostToDevice));
  return NB_OK;
}

int operator_from(Operator *op, int nelx, int nely, int nelz, int nelt, int lx,
                  const int *lglel, const double *dxm1, const GsHost &maps,
                  int mask_mode, cudaStream_t s) {
  NB_TRY(operator_base(op, nelx, nely, nelz, nelt, lx, lglel, dxm1, mask_mode, s));
  op->gsh_host = maps;
  NB_TRY(gs_upload(op->gsh_host, int(op->n), &op->gs, s));
  build_boundary_groups(op);
  op->mask_built = false;
  if (mask_mode == 1) {
    op->mask_built = true;
    NB_TRY(operator_set_mask(op, full_mask_list(*op)));
  } else {
    NB_TRY(operator_set_mask(op, std::vector<int>()));
  }
  return NB_OK;
}

int operator_box(Operator *op, int nelx, int nely, int nelz, int lx,
                 int mask_mode, cudaStream_t s) {
  if (nelx <= 0 || nely <= 0 || nelz <= 0)
    return fail(NB_ERR_ARG, "box %dx%dx%d must be positive", nelx, nely, nelz);
  const long nelt = long(nelx) * nely * nelz;
  if (nelt * lx * lx * lx >= (1L << 31))
    return fail(NB_ERR_UNSUPPORTED, "n = nelt*lx1^3 = %ld exceeds 2^31-1",
                nelt * lx * lx * lx);
  std::vector<int> lglel(nelt);
  for (long e = 0; e < nelt; ++e) lglel[e] = int(e + 1);  // brick, np=1
  std::vector<double> a(lx * lx), b(lx), c(lx * lx), d(lx * lx), z(lx);
  semhat(a.data(), b.data(), c.data(), d.data(), z.data(), lx - 1);
  if (setup_on_device()) {
    NB_TRY(operator_base(op, nelx, nely, nelz, int(nelt), lx, lglel.data(), d.data(),
                         mask_mode, s));
    return box_topology_device(op, s);
  }
  const long n = nelt * lx * lx * lx;
  std::vector<int64_t> glo(n);
  set_vert_box(glo.data(), lx, int(nelt), nelx, nely, lglel.data());
  GsHost maps;
  gs_topology(glo.data(), int(n), &maps);
  NB_TRY(operator_from(op, nelx, nely, nelz, int(nelt), lx, lglel.data(), d.data(), maps,
                       mask_mode, s));
  op->brick = true;
  return NB_OK;
}

// ------------------------------------------------------- vector kernels --
namespace {

template <typename T>
__global__ void k_add2s1(T *a, const T *b, const double *c1d, double c1h, long n) {
  const T c1 = T(c1d ? *c1d : c1h);
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = fma_rn(c1, a[q], b[q]);
}
template <typename T>
__global__ void k_add2s2(T *a, const T *b, T c1, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = fma_rn(c1, b[q], a[q]);
}
template <typename T>
__global__ void k_copy_first(T *p, const T *z, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    p[q] = z[q];
}
template <typename T, typename S>
__global__ void k_convert(T *a, const S *b, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = T(b[q]);
}
template <typename T>
__global__ void k_mask_list(T *w, const int *list, int nlist) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nlist) w[list[q]] = T(0);
}
// zero every element's domain faces (the build branch of maskit, cg.f:236-250)
template <typename T>
__global__ void k_mask_faces(T *w, const unsigned char *face, int lx, long n) {
  const long l3 = long(lx) * lx * lx;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x) {
    const unsigned f = face[q / l3];
    if (!f) continue;
    const int r = int(q % l3);
    const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
    if (((f & 1u) && i == 0) || ((f & 2u) && i == lx - 1) || ((f & 4u) && j == 0) ||
        ((f & 8u) && j == lx - 1) || ((f & 16u) && k == 0) || ((f & 32u) && k == lx - 1))
      w[q] = T(0);
  }
}
// pap = glsc3(w,c,p), alpha = rtz1/pap (unfused path)
__global__ void k_set_alpha(CgScalars *sc, const double *pap) {
  sc->pap = *pap;
  sc->alpha = sc->rtz1 / *pap;
}

int grid_for(long n) {
  return int(std::max(1L, std::min<long>(long(sm_count()) * 8, (n + 255) / 256)));
}

// Each element's face bits (cface: bit 0/1 the faces i = 0 / lx-1 have a
// neighbour, 2/3 for j, 4/5 for k; read from c at the face points (1,1),
// 1/2 with a neighbour), and *ok cleared when any point's c differs
// bitwise from 2^-m, m the number of its extreme local indices on faces
// with a neighbour (lx >= 3).  One block per element at a time.
__global__ void k_c_closed_form(const float *__restrict__ c, int lx, long nelt,
                                unsigned char *__restrict__ cface, int *ok) {
  __shared__ unsigned fb_s;
  const int L2 = lx * lx, L3 = L2 * lx;
  for (long e = blockIdx.x; e < nelt; e += gridDim.x) {
    const float *ce = c + e * L3;
    if (threadIdx.x == 0) {
      const int m = 1, h = lx - 1;
      const int pt[6] = {0 + lx * m + L2 * m, h + lx * m + L2 * m, m + 0 + L2 * m,
                         m + lx * h + L2 * m, m + lx * m + 0,  m + lx * m + L2 * h};
      unsigned fb = 0;
      for (int f = 0; f < 6; ++f)
        if (ce[pt[f]] == 0.5f) fb |= 1u << f;
      fb_s = fb;
      cface[e] = (unsigned char)fb;
    }
    __syncthreads();
    const unsigned fb = fb_s;
    bool good = true;
    for (int l = threadIdx.x; l < L3; l += blockDim.x) {
      const int i = l % lx, j = (l / lx) % lx, k = l / L2;
      const unsigned b = (i == 0 ? 1u : 0u) | (i == lx - 1 ? 2u : 0u) | (j == 0 ? 4u : 0u) |
                         (j == lx - 1 ? 8u : 0u) | (k == 0 ? 16u : 0u) |
                         (k == lx - 1 ? 32u : 0u);
      const unsigned want = unsigned(127 - __popc(b & fb)) << 23;
      good &= __float_as_uint(ce[l]) == want;
    }
    // (also keeps the next element's fb_s write behind every read of this one)
    if (!__syncthreads_and(good) && threadIdx.x == 0) atomicExch(ok, 0);
  }
}

}  // namespace

int c_closed_form(const Operator &op, const float *c32, unsigned char *cface, int *flag,
                  bool *closed, cudaStream_t s) {
  *closed = false;
  if (op.lx % 2 != 0 || op.lx < 4 || op.lx > 16 || op.nelt < 1) return NB_OK;
  const int one = 1;
  int h = 0;
  NB_CUDA(cudaMemcpyAsync(flag, &one, sizeof(int), cudaMemcpyHostToDevice, s));
  const int grid = int(std::min<long>(op.nelt, long(sm_count()) * 8));
  k_c_closed_form<<<grid, 256, 0, s>>>(c32, op.lx, op.nelt, cface, flag);
  NB_CUDA(cudaGetLastError());
  NB_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  NB_CUDA(cudaStreamSynchronize(s));
  *closed = h != 0;
  return NB_OK;
}

namespace {
// k_cg_update with pairing mode D; FP32 forms c in closed form when the
// solve in progress verified it (wk.c32_face)
template <typename T, int D>
void update_launch(const Operator &op, const CgWork &wk, T *x, T *r, const T *p,
                   const T *w, const T *c, double *hist, int iter, int identity,
                   float *r32, const T *pprev, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    if (wk.c32_face) {
      k_cg_update<T, D, true><<<wk.grid_up, 256, 0, s>>>(
          x, r, p, w, c, op.n, wk.partial_up, wk.counters + 1, wk.sc, hist, iter, identity,
          r32, pprev, wk.c32_face, op.lx);
      return;
    }
  }
  k_cg_update<T, D><<<wk.grid_up, 256, 0, s>>>(x, r, p, w, c, op.n, wk.partial_up,
                                               wk.counters + 1, wk.sc, hist, iter, identity,
                                               r32, pprev);
}
}  // namespace

template <typename T>
int vec_add2s1(T *a, const T *b, const double *c1d, double c1, long n, cudaStream_t s) {
  k_add2s1<T><<<grid_for(n), 256, 0, s>>>(a, b, c1d, c1, n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}
template <typename T>
int vec_add2s2(T *a, const T *b, double c1, long n, cudaStream_t s) {
  k_add2s2<T><<<grid_for(n), 256, 0, s>>>(a, b, T(c1), n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}
template <typename T>
int vec_mask(T *w, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return NB_OK;
  k_mask_list<T><<<(nlist + 255) / 256, 256, 0, s>>>(w, list, nlist);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}
template <typename T>
int vec_copy(T *a, const T *b, long n, cudaStream_t s) {
  NB_CUDA(cudaMemcpyAsync(a, b, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
  return NB_OK;
}
template <typename T, typename S>
int vec_convert(T *a, const S *b, long n, cudaStream_t s) {
  k_convert<T, S><<<grid_for(n), 256, 0, s>>>(a, b, n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}
template <typename T>
int vec_glsc3(const T *a, const T *b, const T *m, long n, CgWork &wk,
              double *out, CgScalars *sc, int mode, int iter, cudaStream_t s,
              const float *mf, T *mout) {
  const int gr = std::min(grid_for(n), wk.grid_up);
  k_glsc3<T><<<gr, 256, 0, s>>>(a, b, m, n, wk.partial_dot, wk.counters + 2, out,
                                sc, mode, wk.hist, iter, mf, mout);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

template int vec_add2s1<double>(double *, const double *, const double *, double, long, cudaStream_t);
template int vec_add2s1<float>(float *, const float *, const double *, double, long, cudaStream_t);
template int vec_add2s2<double>(double *, const double *, double, long, cudaStream_t);
template int vec_add2s2<float>(float *, const float *, double, long, cudaStream_t);
template int vec_mask<double>(double *, const int *, int, cudaStream_t);
template int vec_mask<float>(float *, const int *, int, cudaStream_t);
template int vec_copy<double>(double *, const double *, long, cudaStream_t);
template int vec_copy<float>(float *, const float *, long, cudaStream_t);
template int vec_convert<float, double>(float *, const double *, long, cudaStream_t);
template int vec_convert<double, float>(double *, const float *, long, cudaStream_t);
template int vec_glsc3<double>(const double *, const double *, const double *, long, CgWork &, double *, CgScalars *, int, int, cudaStream_t, const float *, double *);
template int vec_glsc3<float>(const float *, const float *, const float *, long, CgWork &, double *, CgScalars *, int, int, cudaStream_t, const float *, float *);

// ------------------------------------------------------------ ax launch --
// launch_ax<T> is instantiated in nb_ax_f64.cu / nb_ax_f32.cu (one
// translation unit per precision and mode, so the builds run in parallel).

// maskit (cg.f:214-258) on a device vector: the build branch (zero every
// element's domain faces, then record element 1's zero entries) on the first
// call after a reset in reference mode, the recorded list otherwise.
template <typename T>
static int maskit_dev(Operator &op, T *w, cudaStream_t s) {
  if (op.mask_mode == 0 && !op.mask_built) {
    k_mask_faces<T><<<grid_for(op.n), 256, 0, s>>>(w, op.d_face, op.lx, op.n);
    NB_CUDA(cudaGetLastError());
    const int l3 = op.lx * op.lx * op.lx;
    std::vector<T> e1(l3);
    NB_CUDA(cudaMemcpyAsync(e1.data(), w, l3 * sizeof(T), cudaMemcpyDeviceToHost, s));
    NB_CUDA(cudaStreamSynchronize(s));
    std::vector<int> list;
    for (int i = 0; i < l3; ++i)
      if (e1[i] == T(0)) list.push_back(i);
    op.mask_built = true;
    return operator_set_mask(&op, list);
  }
  return vec_mask<T>(w, op.d_mask_list, op.n_mask, s);
}

template <typename T>
int apply_ax(const Operator &op_c, T *w, const T *u, const T *g, cudaStream_t s) {
  Operator &op = const_cast<Operator &>(op_c);
  AxArgs<T> a{};
  a.w = w;
  a.u = u;
  a.g = g;
  a.D = std::is_same<T, double>::value ? (const T *)op.dD : (const T *)op.fD;
  NB_TRY(launch_ax<T>(op, 0, a, s));
  NB_TRY(gs_exec(op.gs, w, std::is_same<T, double>::value ? 1 : 2, 1, 0, s));
  NB_TRY(vec_add2s2<T>(w, u, 0.1, op.n, s));
  return maskit_dev<T>(op, w, s);
}
template int apply_ax<double>(const Operator &, double *, const double *, const double *, cudaStream_t);
template int apply_ax<float>(const Operator &, float *, const float *, const float *, cudaStream_t);

// ------------------------------------------------------------------ CG --
// cg.f:36-42: x = 0, r = mask(f), rnorm = sqrt(glsc3(r,c,r)).
template <typename T>
static int cg_begin_t(Operator &op, CgWork &wk, T *x, const T *f, const T *c,
                      T *r, bool zero_x, int niter, cudaStream_t s) {
  const long n = op.n;
  NB_TRY(wk.ensure(op, niter));
  wk.r32_ready = false;
  if (std::is_same<T, double>::value) metric_fx_invalidate(op);
  if (zero_x) NB_CUDA(cudaMemsetAsync(x, 0, n * sizeof(T), s));  // rzero(x)
  NB_TRY(vec_copy<T>(r, f, n, s));                                 // copy(r,f)
  NB_TRY(maskit_dev<T>(op, r, s));
  return vec_glsc3<T>(r, c, r, n, wk, wk.dot_out, wk.sc, 1, 0, s);
}

// iterations it0..it1 of cg.f:48-75.  With p_alt (the fused, unpreconditioned
// iteration), the directions of odd iterations go to p and those of even
// iterations to p_alt, and each pair (odd, even) of iterations inside
// it0..it1 updates x once (k_cg_update DEFER 1, then 2); the direction of
// an even last iteration stays in p_alt (cg_device copies it to p).
template <typename T>
static int cg_steps_t(Operator &op, CgWork &wk, T *x, const T *g, const T *c,
                      T *r, T *w, T *p, T *z, int it0, int it1, int niter,
                      Precond *M, bool force_unfused, cudaStream_t s,
                      T *p_alt = nullptr) {
  const long n = op.n;
  const T *D = std::is_same<T, double>::value ? (const T *)op.dD : (const T *)op.fD;
  const bool tc = std::is_same<T, float>::value && wk.tc_inner;
  const bool fused = op.fused_ok && !force_unfused && !tc;
  const bool paired = p_alt && fused && !M;
  T *const p_odd = p;
  for (int iter = it0; iter <= it1; ++iter) {
    T *pold = nullptr;
    if (paired) {
      p = (iter & 1) ? p_odd : p_alt;
      pold = (iter & 1) ? p_alt : p_odd;
    }
    T *zz = r;
    if (M) {
      if (!std::is_same<T, double>::value)
        return fail(NB_ERR_UNSUPPORTED, "preconditioned CG is FP64 only");
      zz = z;
      if (wk.r32_ready && M->r32_in()) {
        // the update already wrote float(r); z arrives in FP32 and becomes
        // FP64 inside glsc3(r, c, z) (same values as the conversion passes)
        NB_TRY(M->apply_f32(s));
        NB_TRY(vec_glsc3<T>(r, c, z, n, wk, wk.dot_out + 1, wk.sc, 2, iter, s,
                            M->z32_out(), z));
      } else {
        NB_TRY(M->apply((double *)z, (double *)r, s));
        NB_TRY(vec_glsc3<T>(r, c, z, n, wk, wk.dot_out + 1, wk.sc, 2, iter, s));
      }
    } else if (z && z != r && iter == niter) {
      // hsmg_dum's solveM leaves z = r of the last iteration (hsmg_dum.f:9-14)
      NB_TRY(vec_copy<T>(z, r, n, s));
    }
    if (fused) {
      AxArgs<T> a{};
      a.w = w;
      a.u = zz;
      a.p = p;
      a.g = g;
      a.c = c;
      a.D = D;
      a.sc = wk.sc;
      a.partial = wk.partial_ax;
      a.first = iter == 1;
      a.pold = iter == 1 ? nullptr : pold;
      a.c_unit_interior = std::is_same<T, float>::value && wk.c32_face ? 1 : 0;
      a.g_uniform = std::is_same<T, float>::value ? wk.g32_uniform : 0;
      NB_TRY(launch_ax<T>(op, 1, a, s));
      k_gs_fin<T><<<wk.grid_gs, 256, 0, s>>>(w, p, c, op.bnd_off, op.bnd_idx,
                                             op.nbg, wk.partial_gs, wk.partial_ax,
                                             op.nelt, wk.counters + 0, wk.sc);
      NB_CUDA(cudaGetLastError());
    } else {
      if (iter == 1)
        k_copy_first<T><<<grid_for(n), 256, 0, s>>>(p, zz, n);
      else
        NB_TRY(vec_add2s1<T>(p, zz, &wk.sc->beta, 0.0, n, s));
      if constexpr (std::is_same<T, float>::value) {
        if (tc) NB_TRY(apply_ax_tc(op, w, p, g, s));
        else NB_TRY(apply_ax<T>(op, w, p, g, s));
      } else {
        NB_TRY(apply_ax<T>(op, w, p, g, s));
      }
      NB_TRY(vec_glsc3<T>(w, c, p, n, wk, wk.dot_out + 2, nullptr, 0, iter, s));
      k_set_alpha<<<1, 1, 0, s>>>(wk.sc, wk.dot_out + 2);
      NB_CUDA(cudaGetLastError());
    }
    float *r32 = M ? M->r32_in() : nullptr;
    double *hist = iter < wk.hist_len ? wk.hist : nullptr;
    if (paired && (iter & 1) && iter < it1)
      update_launch<T, 1>(op, wk, x, r, p, w, c, hist, iter, 1, nullptr, nullptr, s);
    else if (paired && !(iter & 1) && iter > it0)
      update_launch<T, 2>(op, wk, x, r, p, w, c, hist, iter, 1, nullptr, pold, s);
    else
      update_launch<T, 0>(op, wk, x, r, p, w, c, hist, iter, M == nullptr, r32, nullptr, s);
    wk.r32_ready = r32 != nullptr;
    NB_CUDA(cudaGetLastError());
  }
  return NB_OK;
}

// x += scale*e; r = f - A x; rtr -> sc (MODE 2 + k_gs_res)
int residual_fused(Operator &op, CgWork &wk, double *x, const float *e,
                   double scale, const double *f, const double *g,
                   const double *c, double *r, double *w, cudaStream_t s) {
  NB_TRY(wk.ensure(op, 1));
  AxArgs<double> a{};
  a.w = w;
  a.p = x;
  a.g = g;
  a.c = c;
  a.D = op.dD;
  a.sc = wk.sc;
  a.partial = wk.partial_ax;
  a.f = f;
  a.r = r;
  a.e = e;
  a.scale = scale;
  NB_TRY(launch_ax<double>(op, 2, a, s));
  k_gs_res<double><<<wk.grid_gs, 256, 0, s>>>(w, x, f, r, c, op.bnd_off, op.bnd_idx,
                                              op.nbg, wk.partial_gs, wk.partial_ax,
                                              op.nelt, wk.counters + 0, wk.sc);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

template <typename T>
int time_cg_kernels_t(Operator &op, CgWork &wk, T *x, const T *f, const T *g,
                      const T *c, T *r, T *w, T *p, int reps, double *ms3,
                      cudaStream_t s) {
  // the solvers' forms: directions alternating between p and a second
  // buffer, x updated once per pair of iterations (nb_set_paired_update),
  // and for FP32 c formed in closed form where it verifies
  // (nb_set_mixed_closed_multiplicity)
  const bool PAIRED = g_paired_update;
  constexpr bool F32 = std::is_same<T, float>::value;
  const int iters = PAIRED ? 2 * reps : reps;
  T *p_alt = nullptr;
  unsigned char *cface = nullptr;
  std::unique_ptr<T, int (*)(T *)> p_alt_owner(nullptr, [](T *q) { return int(cudaFree(q)); });
  std::unique_ptr<unsigned char, int (*)(unsigned char *)> cface_owner(
      nullptr, [](unsigned char *q) { return int(cudaFree(q)); });
  if (PAIRED) {
    NB_CUDA(cudaMalloc(&p_alt, op.n * sizeof(T)));
    p_alt_owner.reset(p_alt);
  }
  if (F32 && g_mixed_closed_c) {
    NB_CUDA(cudaMalloc(&cface, size_t(op.nelt) + 16));
    cface_owner.reset(cface);
  }
  struct FaceReset {
    CgWork &wk;
    ~FaceReset() { wk.c32_face = nullptr; }
  } face_reset{wk};
  if constexpr (F32) {
    if (cface) {
      bool closed = false;
      int *flag = reinterpret_cast<int *>(cface + ((size_t(op.nelt) + 3) & ~size_t(3)));
      NB_TRY(c_closed_form(op, (const float *)c, cface, flag, &closed, s));
      wk.c32_face = closed ? cface : nullptr;
    }
  }
  NB_TRY(cg_begin_t<T>(op, wk, x, f, c, r, true, iters + 2, s));
  NB_TRY(cg_steps_t<T>(op, wk, x, g, c, r, w, p, r, 1, 1, -1, nullptr, false, s));
  cudaEvent_t ev[4];
  for (auto &e : ev) NB_CUDA(cudaEventCreate(&e));
  double acc[3] = {0, 0, 0};
  const T *D = std::is_same<T, double>::value ? (const T *)op.dD : (const T *)op.fD;
  for (int it = 0; it < iters; ++it) {
    // iteration it + 2; pairs (2,3), (4,5), ...: the first of a pair writes
    // its direction to p_alt and defers its x update
    const bool first_of_pair = PAIRED && (it & 1) == 0;
    T *pc = first_of_pair ? p_alt : p;
    const T *po = !PAIRED ? nullptr : first_of_pair ? p : p_alt;
    AxArgs<T> a{};
    a.w = w;
    a.u = r;
    a.p = pc;
    a.pold = po;
    a.g = g;
    a.c = c;
    a.c_unit_interior = wk.c32_face ? 1 : 0;
    a.D = D;
    a.sc = wk.sc;
    a.partial = wk.partial_ax;
    NB_CUDA(cudaEventRecord(ev[0], s));
    NB_TRY(launch_ax<T>(op, 1, a, s));
    NB_CUDA(cudaEventRecord(ev[1], s));
    k_gs_fin<T><<<wk.grid_gs, 256, 0, s>>>(w, pc, c, op.bnd_off, op.bnd_idx, op.nbg,
                                           wk.partial_gs, wk.partial_ax, op.nelt,
                                           wk.counters + 0, wk.sc);
    NB_CUDA(cudaEventRecord(ev[2], s));
    if (!PAIRED)
      update_launch<T, 0>(op, wk, x, r, pc, w, c, nullptr, it + 2, 1, nullptr, nullptr, s);
    else if (first_of_pair)
      update_launch<T, 1>(op, wk, x, r, pc, w, c, nullptr, it + 2, 1, nullptr, nullptr, s);
    else
      update_launch<T, 2>(op, wk, x, r, pc, w, c, nullptr, it + 2, 1, nullptr, po, s);
    NB_CUDA(cudaEventRecord(ev[3], s));
    NB_CUDA(cudaEventSynchronize(ev[3]));
    for (int k = 0; k < 3; ++k) {
      float ms = 0;
      NB_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
      acc[k] += ms;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  for (int k = 0; k < 3; ++k) ms3[k] = acc[k] / (iters > 0 ? iters : 1);
  return NB_OK;
}
template int time_cg_kernels_t<double>(Operator &, CgWork &, double *, const double *,
                                       const double *, const double *, double *, double *,
                                       double *, int, double *, cudaStream_t);
template int time_cg_kernels_t<float>(Operator &, CgWork &, float *, const float *,
                                      const float *, const float *, float *, float *,
                                      float *, int, double *, cudaStream_t);

int launch_gs_fin(const Operator &op, CgWork &wk, double *w, const double *p,
                  const double *c, cudaStream_t s) {
  k_gs_fin<double><<<wk.grid_gs, 256, 0, s>>>(w, p, c, op.bnd_off, op.bnd_idx,
                                              op.nbg, wk.partial_gs, wk.partial_ax,
                                              op.nelt, wk.counters + 0, wk.sc);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

int launch_cg_update(const Operator &op, CgWork &wk, double *x, double *r,
                     const double *p, const double *w, const double *c,
                     int iter, cudaStream_t s) {
  k_cg_update<double><<<wk.grid_up, 256, 0, s>>>(x, r, p, w, c, op.n, wk.partial_up,
                                                 wk.counters + 1, wk.sc, nullptr,
                                                 iter, 1);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

int cg_device(Operator &op, CgWork &wk, double *x, const double *f,
              const double *g, const double *c, double *r, double *w,
              double *p, double *z, int niter, Precond *M, bool force_unfused,
              cudaStream_t s) {
  NB_TRY(cg_begin_t<double>(op, wk, x, f, c, r, true, niter, s));
  // the second direction buffer of the paired x update (fused, no
  // preconditioner, at least one pair)
  double *p_alt = nullptr;
  if (g_paired_update && !M && !force_unfused && op.fused_ok && niter >= 2) {
    NB_TRY(wk.ensure_palt(op.n));
    p_alt = wk.palt;
  }
  NB_TRY(cg_steps_t<double>(op, wk, x, g, c, r, w, p, z, 1, niter, niter, M,
                            force_unfused, s, p_alt));
  // the last direction is the caller's p (cg.f's p on return)
  if (p_alt && niter % 2 == 0)
    NB_CUDA(cudaMemcpyAsync(p, p_alt, op.n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return NB_OK;
}

int cg_begin(Operator &op, CgWork &wk, double *x, const double *f,
             const double *c, double *r, int niter, cudaStream_t s) {
  return cg_begin_t<double>(op, wk, x, f, c, r, true, niter, s);
}

int cg_steps(Operator &op, CgWork &wk, double *x, const double *g,
             const double *c, double *r, double *w, double *p, int it0,
             int it1, cudaStream_t s) {
  return cg_steps_t<double>(op, wk, x, g, c, r, w, p, r, it0, it1, -1, nullptr,
                            false, s);
}

int cg_steps_pc(Operator &op, CgWork &wk, double *x, const double *g,
                const double *c, double *r, double *w, double *p, double *z,
                int it0, int it1, Precond *M, cudaStream_t s) {
  return cg_steps_t<double>(op, wk, x, g, c, r, w, p, z, it0, it1, -1, M, false, s);
}

int cg_device_f32(Operator &op, CgWork &wk, float *x, const float *f,
                  const float *g, const float *c, float *r, float *w, float *p,
                  int niter, cudaStream_t s, float *p_alt) {
  NB_TRY(cg_begin_t<float>(op, wk, x, f, c, r, true, niter, s));
  return cg_steps_t<float>(op, wk, x, g, c, r, w, p, r, 1, niter, niter,
                           nullptr, false, s, p_alt);
}

}  // namespace nb

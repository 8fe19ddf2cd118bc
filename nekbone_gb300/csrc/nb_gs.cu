// nb_gs.cu -- the jl gather-scatter (gs_op) on the GPU.
//
// Semantics follow gs_aux (jl/gs.c:1029-1045) at one process: gather over the
// unflagged map (gather_T_OP, jl/gs_local.c:60-75), set flagged primaries to
// the operation's identity (init_T, gs_local.c:88-94), scatter over the full
// map (scatter_T, gs_local.c:77-86); transpose swaps the two maps and skips
// the init.  The remote exchange is empty with one process.
//
// Device layout: each map is stored as CSR (offsets + members, primary first,
// members in jl's order), so one thread owns one group and reproduces jl's
// summation order exactly: t = u[primary]; t op= u[m] for each member in map
// order.  Groups are ordered by ascending primary, as jl orders them.
#include <float.h>
#include <limits.h>

#include "nb_internal.h"

namespace nb {

namespace {

template <typename T>
struct Ident;
template <>
struct Ident<double> {
  __device__ static double mx() { return DBL_MAX; }
  __device__ static double mn() { return -DBL_MAX; }
};
template <>
struct Ident<float> {
  __device__ static float mx() { return FLT_MAX; }
  __device__ static float mn() { return -FLT_MAX; }
};
template <>
struct Ident<int> {
  __device__ static int mx() { return INT_MAX; }
  __device__ static int mn() { return INT_MIN; }
};
template <>
struct Ident<long long> {
  __device__ static long long mx() { return LLONG_MAX; }
  __device__ static long long mn() { return LLONG_MIN; }
};

// op: 1 add, 2 mul, 3 min, 4 max (GS_DO_*, jl/gs_defs.h:35-38)
template <typename T, int OP>
__device__ __forceinline__ void gs_do(T &a, T b) {
  if (OP == 1) a += b;
  if (OP == 2) a *= b;
  if (OP == 3) {
    if (b < a) a = b;
  }
  if (OP == 4) {
    if (b > a) a = b;
  }
}

template <typename T, int OP>
__device__ __forceinline__ T gs_identity() {
  if (OP == 1) return T(0);
  if (OP == 2) return T(1);
  if (OP == 3) return Ident<T>::mx();
  return Ident<T>::mn();
}

// Symmetric fast path: gather and scatter over the same groups.
template <typename T, int OP>
__global__ void k_gs_sym(T *__restrict__ u, const int *__restrict__ off,
                         const int *__restrict__ idx, int ng) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int b = off[g], e = off[g + 1];
    T t = u[idx[b]];
    for (int q = b + 1; q < e; ++q) gs_do<T, OP>(t, u[idx[q]]);
    for (int q = b; q < e; ++q) u[idx[q]] = t;
  }
}

template <typename T, int OP>
__global__ void k_gs_gather(T *__restrict__ u, const int *__restrict__ off,
                            const int *__restrict__ idx, int ng) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int b = off[g], e = off[g + 1];
    T t = u[idx[b]];
    for (int q = b + 1; q < e; ++q) gs_do<T, OP>(t, u[idx[q]]);
    u[idx[b]] = t;
  }
}

template <typename T>
__global__ void k_gs_scatter(T *__restrict__ u, const int *__restrict__ off,
                             const int *__restrict__ idx, int ng) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int b = off[g], e = off[g + 1];
    const T t = u[idx[b]];
    for (int q = b + 1; q < e; ++q) u[idx[q]] = t;
  }
}

template <typename T, int OP>
__global__ void k_gs_init(T *__restrict__ u, const int *__restrict__ fp,
                          int nfp) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nfp) u[fp[g]] = gs_identity<T, OP>();
}

// jl map -> CSR
void map_to_csr(const std::vector<uint32_t> &map, std::vector<int> &off,
                std::vector<int> &idx) {
  const uint32_t END = uint32_t(-1);
  off.clear();
  idx.clear();
  size_t p = 0;
  while (p < map.size() && map[p] != END) {
    off.push_back(int(idx.size()));
    idx.push_back(int(map[p++]));
    while (map[p] != END) idx.push_back(int(map[p++]));
    ++p;
  }
  off.push_back(int(idx.size()));
}

int upload_ints(const std::vector<int> &h, int **d, cudaStream_t s) {
  *d = nullptr;
  if (h.empty()) return NB_OK;
  NB_CUDA(cudaMalloc(d, h.size() * sizeof(int)));
  NB_CUDA(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(int),
                          cudaMemcpyHostToDevice, s));
  return NB_OK;
}

inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

// The grid of a grid-stride gather-scatter kernel: the blocks the SMs hold
// at once (one wave), or fewer when there are fewer groups -- the launch
// shape that made the fused boundary pass (k_gs_fin) fastest.  For these
// passes it measured the same as one group per thread (hsmg's V-cycle, the
// unfused operator at 16^3).
template <typename K>
int resident_blocks(K kernel, int tb) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, tb, 0);
  return std::max(1, sms) * std::max(1, per_sm);
}
template <typename T, int OP>
int sym_grid(int ng) {
  static const int cap = resident_blocks(k_gs_sym<T, OP>, 256);
  return std::min(blocks_for(ng, 256), cap);
}
template <typename T, int OP>
int gather_grid(int ng) {
  static const int cap = resident_blocks(k_gs_gather<T, OP>, 256);
  return std::min(blocks_for(ng, 256), cap);
}
template <typename T>
int scatter_grid(int ng) {
  static const int cap = resident_blocks(k_gs_scatter<T>, 256);
  return std::min(blocks_for(ng, 256), cap);
}

template <typename T, int OP>
void run_gs(const GsDevice &d, T *u, int transpose, cudaStream_t s) {
  const int TB = 256;
  if (d.symmetric) {
    if (d.ng > 0)
      k_gs_sym<T, OP><<<sym_grid<T, OP>(d.ng), TB, 0, s>>>(u, d.off, d.idx, d.ng);
    return;
  }
  const int *og = transpose ? d.off_s : d.off_g, *ig = transpose ? d.idx_s : d.idx_g;
  const int ngg = transpose ? d.ng_s : d.ng_g;
  const int *os = transpose ? d.off_g : d.off_s, *is = transpose ? d.idx_g : d.idx_s;
  const int ngs = transpose ? d.ng_g : d.ng_s;
  if (ngg > 0) k_gs_gather<T, OP><<<gather_grid<T, OP>(ngg), TB, 0, s>>>(u, og, ig, ngg);
  if (!transpose && d.nfp > 0)
    k_gs_init<T, OP><<<blocks_for(d.nfp, TB), TB, 0, s>>>(u, d.fprim, d.nfp);
  if (ngs > 0) k_gs_scatter<T><<<scatter_grid<T>(ngs), TB, 0, s>>>(u, os, is, ngs);
}

template <typename T>
int run_gs_op(const GsDevice &d, T *u, int op, int transpose, cudaStream_t s) {
  switch (op) {
    case 1: run_gs<T, 1>(d, u, transpose, s); break;
    case 2: run_gs<T, 2>(d, u, transpose, s); break;
    case 3: run_gs<T, 3>(d, u, transpose, s); break;
    case 4: run_gs<T, 4>(d, u, transpose, s); break;
    default: return fail(NB_ERR_ARG, "gs_op: op %d not in valid range 1-4", op);
  }
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

}  // namespace

int gs_upload(const GsHost &h, int n, GsDevice *d, cudaStream_t s) {
  *d = GsDevice();
  d->n = n;
  d->symmetric = (h.map[0] == h.map[1]) && h.map[2].size() == 1;
  std::vector<int> off, idx;
  if (d->symmetric) {
    map_to_csr(h.map[0], off, idx);
    d->ng = int(off.size()) - 1;
    NB_TRY(upload_ints(off, &d->off, s));
    NB_TRY(upload_ints(idx, &d->idx, s));
  } else {
    map_to_csr(h.map[0], off, idx);
    d->ng_g = int(off.size()) - 1;
    NB_TRY(upload_ints(off, &d->off_g, s));
    NB_TRY(upload_ints(idx, &d->idx_g, s));
    map_to_csr(h.map[1], off, idx);
    d->ng_s = int(off.size()) - 1;
    NB_TRY(upload_ints(off, &d->off_s, s));
    NB_TRY(upload_ints(idx, &d->idx_s, s));
    std::vector<int> fp(h.map[2].begin(), h.map[2].end() - 1);
    d->nfp = int(fp.size());
    NB_TRY(upload_ints(fp, &d->fprim, s));
  }
  NB_CUDA(cudaStreamSynchronize(s));
  return NB_OK;
}

void gs_release(GsDevice *d) {
  int *ptrs[] = {d->off, d->idx, d->off_g, d->idx_g, d->off_s, d->idx_s, d->fprim};
  for (int *p : ptrs)
    if (p) cudaFree(p);
  *d = GsDevice();
}

int gs_exec(const GsDevice &d, void *u, int dom, int op, int transpose,
            cudaStream_t s) {
  switch (dom) {
    case 1: return run_gs_op(d, static_cast<double *>(u), op, transpose, s);
    case 2: return run_gs_op(d, static_cast<float *>(u), op, transpose, s);
    case 3: return run_gs_op(d, static_cast<int *>(u), op, transpose, s);
    case 4: return run_gs_op(d, static_cast<long long *>(u), op, transpose, s);
    default:
      return fail(NB_ERR_ARG, "gs_op: datatype %d not in valid range 1-4", dom);
  }
}

}  // namespace nb

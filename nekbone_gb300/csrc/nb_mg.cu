// nb_mg.cu -- hybrid Schwarz multigrid preconditioner (hsmg.f) on the GPU.
//
// h1mg_solve (hsmg.f:960-1034) is an additive V-cycle: an overlapping
// Schwarz smoother on every level but the coarsest, weighted restriction
// down, a "coarse solve" that is a copy plus dssum (hsmg_coarse_solve,
// hsmg.f:945-957), and interpolation back up with no post-smoothing.  The
// Schwarz step (h1mg_schwarz_part1, hsmg.f:1053-1095) works on elements
// extended by one ghost layer: ghost faces receive the neighbour's first
// interior layer through a gather-scatter on the extended numbering, each
// extended element is solved by fast diagonalisation (h1mg_do_fast,
// hsmg.f:1297-1318), and the overlapping contributions are summed back.
// Every tensor apply is the reference's three mxm passes (h1mg_tnsr3d_el,
// hsmg.f:1320-1338) with left-to-right sums.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <tuple>

#include "nb_mg.h"

namespace nb {

Multigrid::~Multigrid() {
  for (int l = 0; l < 8; ++l) {
    MgLevel &L = lv[l];
    gs_release(&L.gs);
    gs_release(&L.gsx);
    double *ps[] = {L.rstr_wt, L.fast_s, L.fast_d, L.schwarz_wt, L.jh, L.jht, L.e, L.r};
    for (double *p : ps)
      if (p) cudaFree(p);
    if (L.mask) cudaFree(L.mask);
    float *pf[] = {L.rstr_wt_f, L.fast_s_f, L.fast_d_f, L.schwarz_wt_f, L.jh_f, L.jht_f,
                   L.e_f, L.r_f};
    for (float *p : pf)
      if (p) cudaFree(p);
  }
  if (A) cudaFree(A);
  if (B) cudaFree(B);
  if (w) cudaFree(w);
  if (A_f) cudaFree(A_f);
  if (B_f) cudaFree(B_f);
  if (z_f) cudaFree(z_f);
  if (c_ainv) cudaFree(c_ainv);
  if (c_gid) cudaFree(c_gid);
  if (c_prim) cudaFree(c_prim);
  if (c_b) cudaFree(c_b);
  if (c_x) cudaFree(c_x);
  if (A2) cudaFree(A2);
  if (B2) cudaFree(B2);
  if (A2_f) cudaFree(A2_f);
  if (B2_f) cudaFree(B2_f);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (s2) cudaStreamDestroy(s2);
}

namespace {

// ---------------------------------------------------------------- device --
// v(nv^3) = [Ct (x) Bt (x) A] u(nu^3): work = A u, work2 = work Bt per slab,
// v = work2 Ct.  A is nv x nu, Bt and Ct are nu x nv, column-major.  All
// operands in shared memory, the CTA cooperates; ends with a barrier.
// T is the working precision (FP64, or FP32 for the FP32 smoother).
template <typename T>
__device__ void tensor3(T *v, const T *u, int nv, int nu, const T *A, const T *Bt,
                        const T *Ct, T *work, T *work2) {
  const int t = threadIdx.x, nt = blockDim.x;
  const int nu2 = nu * nu;
  for (int q = t; q < nv * nu2; q += nt) {  // work(a, n p) = sum_m A(a,m) u(m, n p)
    const int a = q % nv, np_ = q / nv;
    T s = mul_rn(A[a], u[np_ * nu]);
    for (int m = 1; m < nu; ++m) s = fma_rn(A[a + m * nv], u[m + np_ * nu], s);
    work[q] = s;
  }
  __syncthreads();
  for (int q = t; q < nv * nv * nu; q += nt) {  // work2(a,b,p) = sum_n work(a,n,p) Bt(n,b)
    const int a = q % nv, b = (q / nv) % nv, p = q / (nv * nv);
    const T *wp = work + nv * nu * p;
    T s = mul_rn(wp[a], Bt[b * nu]);
    for (int n = 1; n < nu; ++n) s = fma_rn(wp[a + n * nv], Bt[n + b * nu], s);
    work2[q] = s;
  }
  __syncthreads();
  for (int q = t; q < nv * nv * nv; q += nt) {  // v(ab, c) = sum_p work2(ab,p) Ct(p,c)
    const int ab = q % (nv * nv), c = q / (nv * nv);
    T s = mul_rn(work2[ab], Ct[c * nu]);
    for (int p = 1; p < nu; ++p) s = fma_rn(work2[ab + p * nv * nv], Ct[p + c * nu], s);
    v[q] = s;
  }
  __syncthreads();
}

template <typename T>
__device__ inline void load_shared(T *dst, const T *src, int n) {
  for (int q = threadIdx.x; q < n; q += blockDim.x) dst[q] = src[q];
}

// ext index helpers: extended element has nl = nh+2 points per direction
__device__ inline int ghost_face(int a, int b, int c, int nl) {
  // returns 0 (not a ghost-face position), else 1 + axis*2 + (high side)
  const int hi = nl - 1;
  const bool ga = (a == 0 || a == hi), gb = (b == 0 || b == hi), gc = (c == 0 || c == hi);
  if (ga && !gb && !gc) return 1 + (a == hi);
  if (gb && !ga && !gc) return 3 + (b == hi);
  if (gc && !ga && !gb) return 5 + (c == hi);
  return 0;
}

// Grid for the line kernels below: one thread per (element, a, b) line of
// n points, the c loop inside, so each thread splits its index once per
// line rather than once per point (32-bit indices: MG vectors stay below
// 2^31 points).  The c loop goes in chunks of kChunk points, all loads of a
// chunk issued before its stores, so that each thread keeps several memory
// requests in flight.
constexpr int kChunk = 4;
int grid_for(long n) { return int(std::max(1L, std::min<long>(152L * 8, (n + 255) / 256))); }
inline int line_grid(int n, int nelt) { return grid_for(long(n) * n * nelt); }

// h1mg_schwarz_toext3d + extrude(A,0,0,A,2,1) (hsmg.f:1075-1077): regular
// points copied into the extended array, each ghost face set to the
// element's own layer-2 value, ghost edges and corners zero.
template <typename T>
__global__ void k_toext(T *A, const T *r, int nh, int nelt) {
  const int nl = nh + 2, nl2 = nl * nl, nh2 = nh * nh, hi = nl - 1;
  const int lines = nl2 * nelt;
  // ghost coordinate 0 reads layer 2, nl-1 reads layer nl-3 (regular index - 1)
  auto src = [&](int x) { return x == 0 ? 1 : (x == hi ? nh - 2 : x - 1); };
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < lines; t += gridDim.x * blockDim.x) {
    const int e = t / nl2, ab = t - e * nl2, a = ab % nl, b = ab / nl;
    const int gab = (a == 0 || a == hi) + (b == 0 || b == hi);
    const T *re = r + e * nh2 * nh + src(a) + nh * src(b);
    T *Ae = A + e * nl2 * nl + ab;
    for (int c0 = 0; c0 < nl; c0 += kChunk) {
      T v[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u) {
        const int c = c0 + u;
        const int g = gab + (c == 0 || c == hi);  // ghost coordinates of the point
        v[u] = c < nl && g <= 1 ? re[nh2 * src(c)] : T(0);
      }
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
        if (c0 + u < nl) Ae[(c0 + u) * nl2] = v[u];
    }
  }
}

// extrude(A,0,1,A,2,-1) (hsmg.f:1079), applied by the FDM kernels as they
// load A: a ghost-face value minus its layer-2 partner.
template <typename T>
__device__ __forceinline__ T ghost_minus_at(const T *Ae, int a, int b, int c, int nl) {
  const int gf = ghost_face(a, b, c, nl);
  const T v = Ae[a + nl * b + nl * nl * c];
  if (!gf) return v;
  if (gf == 1) a = 2; else if (gf == 2) a = nl - 3;
  else if (gf == 3) b = 2; else if (gf == 4) b = nl - 3;
  else if (gf == 5) c = 2; else c = nl - 3;
  return fma_rn(T(-1), Ae[a + nl * b + nl * nl * c], v);
}

// h1mg_do_fast (hsmg.f:1297-1318): B = S (d .* (S^T A')) per extended
// element, A' being A with the ghost-face correction of hsmg.f:1079; also
// saves B's ghost faces into A (the first extrude of the overlap sum,
// hsmg.f:1084: A <- 0*A + B on the ghost faces).
template <typename T>
__global__ void k_fdm(T *B, T *A, const T *s, const T *d, int nl) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  const int nl2 = nl * nl, nl3 = nl2 * nl;
  T *u = sm, *v = u + nl3, *work = v + nl3, *work2 = work + nl3,
    *S = work2 + nl3;  // 6 matrices nl*nl
  const long e = blockIdx.x;
  for (int q = threadIdx.x; q < nl3; q += blockDim.x)
    u[q] = ghost_minus_at(A + e * nl3, q % nl, (q / nl) % nl, q / nl2, nl);
  load_shared(S, s + e * 6L * nl2, 6 * nl2);
  __syncthreads();
  // s(1,2,1)=S_r^T, s(1,1,2)=S_s, s(1,1,3)=S_t
  tensor3<T>(v, u, nl, nl, S + nl2, S + 2 * nl2, S + 4 * nl2, work, work2);
  const T *de = d + e * nl3;
  for (int q = threadIdx.x; q < nl3; q += blockDim.x) u[q] = mul_rn(de[q], v[q]);
  __syncthreads();
  // s(1,1,1)=S_r, s(1,2,2)=S_s^T, s(1,2,3)=S_t^T
  tensor3<T>(v, u, nl, nl, S, S + 3 * nl2, S + 5 * nl2, work, work2);
  for (int q = threadIdx.x; q < nl3; q += blockDim.x) {
    const int a = q % nl, b = (q / nl) % nl, c = q / nl2;
    B[e * nl3 + q] = v[q];
    if (ghost_face(a, b, c, nl)) A[e * nl3 + q] = v[q];
  }
}

// The FDM kernel with the extended size NL known at compile time.  Each of
// the six tensor passes is Out(i, j) = sum_k C(i, k) In(k, j) over one
// element: In is stored [k][j] (slice stride PS, j contiguous), the 1-D
// matrix as C[k][i] (stride IP, i contiguous), and a thread owns a 4 x 4
// tile of outputs, so each k step is two 16-byte shared loads for sixteen
// multiply-adds.  Each pass writes its output already laid out [k'][j'] for
// the next pass's contraction index k'.  Every output is the left-to-right
// sum of tensor3 (first term a product, then fused multiply-adds in k
// order), so the results are bitwise those of the general kernel.
template <typename T, int NL>
struct FdmShape {
  static constexpr int NL2 = NL * NL, NL3 = NL2 * NL;
  static constexpr int PS = (NL2 + 3) & ~3;  // slice stride of the data buffers
  static constexpr int IP = (NL + 3) & ~3;   // row stride of the 1-D matrices
  static constexpr int NIG = IP / 4, NJG = PS / 4, TILES = NIG * NJG;
  static constexpr int THREADS = (TILES + 31) / 32 * 32;
  static constexpr size_t SMEM = sizeof(T) * (2 * size_t(NL) * PS + 6 * size_t(NL) * IP);
};

template <typename T>
struct Vec4 {
  T v[4];
};
__device__ __forceinline__ Vec4<float> ld4(const float *p) {
  const float4 a = *reinterpret_cast<const float4 *>(p);
  return {{a.x, a.y, a.z, a.w}};
}
__device__ __forceinline__ Vec4<double> ld4(const double *p) {
  const double2 a = reinterpret_cast<const double2 *>(p)[0];
  const double2 b = reinterpret_cast<const double2 *>(p)[1];
  return {{a.x, a.y, b.x, b.y}};
}

// one pass; output (i, j) goes to Out[place(j) + i * IS]
template <typename T, int NL, int IS, typename Place>
__device__ __forceinline__ void fdm_pass(T *Out, const T *In, const T *C, Place place) {
  typedef FdmShape<T, NL> F;
  const int t = threadIdx.x;
  if (t < F::TILES) {
    const int i0 = 4 * (t % F::NIG), j0 = 4 * (t / F::NIG);
    T acc[4][4];
    {
      const Vec4<T> c = ld4(C + i0), x = ld4(In + j0);
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = mul_rn(c.v[a], x.v[b]);
    }
#pragma unroll
    for (int k = 1; k < NL; ++k) {
      const Vec4<T> c = ld4(C + k * F::IP + i0), x = ld4(In + k * F::PS + j0);
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma_rn(c.v[a], x.v[b], acc[a][b]);
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + b;
      if (j >= F::NL2) break;
      T *o = Out + place(j) + i0 * IS;
#pragma unroll
      for (int a = 0; a < 4; ++a)
        if (i0 + a < NL) o[a * IS] = acc[a][b];
    }
  }
  __syncthreads();
}

// [Ct (x) Bt (x) A] applied to X (laid out [a][b + NL c]); the result lands
// in Y laid out [c][a + NL b].  X is overwritten.
template <typename T, int NL>
__device__ __forceinline__ void fdm_tensor3(T *X, T *Y, const T *C3) {
  typedef FdmShape<T, NL> F;
  constexpr int PS = F::PS, MS = NL * F::IP;
  // work(a', b + NL c) -> Y[b][a' + NL c]
  fdm_pass<T, NL, 1>(Y, X, C3, [](int j) { return (j % NL) * PS + NL * (j / NL); });
  // work2(a', b', c) from Y[b][a' + NL c] -> X[c][a' + NL b']
  fdm_pass<T, NL, NL>(X, Y, C3 + MS, [](int j) { return (j / NL) * PS + (j % NL); });
  // v(a', b', c') from X[c][a' + NL b'] -> Y[c'][a' + NL b']
  fdm_pass<T, NL, PS>(Y, X, C3 + 2 * MS, [](int j) { return j; });
}

template <typename T, int NL>
__global__ void __launch_bounds__(FdmShape<T, NL>::THREADS)
    k_fdm_fixed(T *B, T *A, const T *s, const T *d) {
  typedef FdmShape<T, NL> F;
  constexpr int NL2 = F::NL2, NL3 = F::NL3, PS = F::PS, IP = F::IP, MS = NL * IP, HI = NL - 1;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *X = reinterpret_cast<T *>(sm_raw), *Y = X + NL * PS, *C = Y + NL * PS;
  const int e = blockIdx.x, nt = blockDim.x;
  const T *Ae = A + e * NL3, *se = s + e * 6 * NL2, *de = d + e * NL3;
  // X[a][b + NL c] = A with extrude(A,0,1,A,2,-1) applied: one thread per
  // (b, c) line, a unrolled.  A ghost-face point (exactly one coordinate on
  // the ghost layer) takes minus its layer-2 partner: along the line for
  // a = 0 / NL-1, else in the partner line (b or c moved to 2 / NL-3).
  for (int t = threadIdx.x; t < NL2; t += nt) {
    const int b = t % NL, c = t / NL;
    const bool gb = b == 0 || b == HI, gc = c == 0 || c == HI;
    const T *line = Ae + NL * t;
    T v[NL];
#pragma unroll
    for (int a = 0; a < NL; ++a) v[a] = line[a];
    if (!gb && !gc) {
      v[0] = fma_rn(T(-1), v[2], v[0]);
      v[HI] = fma_rn(T(-1), v[NL - 3], v[HI]);
    } else if (gb != gc) {
      const int pb = gb ? (b == 0 ? 2 : NL - 3) : b, pc = gc ? (c == 0 ? 2 : NL - 3) : c;
      const T *partner = Ae + NL * (pb + NL * pc);
#pragma unroll
      for (int a = 1; a < HI; ++a) v[a] = fma_rn(T(-1), partner[a], v[a]);
    }
#pragma unroll
    for (int a = 0; a < NL; ++a) X[a * PS + t] = v[a];
  }
  // the 1-D matrices as C[k][i]: s(1,2,1), s(1,1,2), s(1,1,3) for the first
  // apply (A, Bt, Ct of tensor3), s(1,1,1), s(1,2,2), s(1,2,3) for the second
  for (int q = threadIdx.x; q < 6 * MS; q += nt) {
    const int m = q / MS, r = q - m * MS, k = r / IP, i = r - k * IP;
    const int src = m == 0 ? 1 : m == 1 ? 2 : m == 2 ? 4 : m == 3 ? 0 : m == 4 ? 3 : 5;
    const T *S = se + src * NL2;
    const bool slot_a = m == 0 || m == 3;  // the A slot: C(i,k) = S[i + k NL]
    C[q] = i < NL ? (slot_a ? S[i + k * NL] : S[k + i * NL]) : T(0);
  }
  __syncthreads();
  fdm_tensor3<T, NL>(X, Y, C);
  // d .* v, from Y[c][a + NL b] back to X[a][b + NL c], one (b, c) line each
  for (int t = threadIdx.x; t < NL2; t += nt) {
    const int b = t % NL, c = t / NL;
    const T *yl = Y + c * PS + NL * b, *dl = de + NL * t;
#pragma unroll
    for (int a = 0; a < NL; ++a) X[a * PS + t] = mul_rn(dl[a], yl[a]);
  }
  __syncthreads();
  fdm_tensor3<T, NL>(X, Y, C + 3 * MS);
  // B = v; Y[c][a + NL b] is the natural order with slices PS apart
  T *Be = B + e * NL3;
  for (int q = threadIdx.x; q < NL3; q += nt) Be[q] = Y[(q / NL2) * PS + q % NL2];
  // ghost faces of v into A: face f = 2 axis + side, (x, y) its interior point
  constexpr int NF = (NL - 2) * (NL - 2);
  T *Aw = A + e * NL3;
  for (int q = threadIdx.x; q < 6 * NF; q += nt) {
    const int f = q / NF, r = q - f * NF, x = r % (NL - 2) + 1, y = r / (NL - 2) + 1;
    const int g = (f & 1) ? HI : 0;
    const int a = f < 2 ? g : x, b = f < 2 ? x : (f < 4 ? g : y), c = f < 4 ? y : g;
    Aw[a + NL * b + NL2 * c] = Y[c * PS + a + NL * b];
  }
}

bool g_fixed_kernels = true;

// The fixed-size FDM kernel for an extended size nl (5..18), else null
template <typename T>
using FdmFn = void (*)(T *, T *, const T *, const T *);
template <typename T>
FdmFn<T> fdm_fixed_any(int nl) {
  switch (nl) {
#define NB_FDM(N) \
  case N: return k_fdm_fixed<T, N>;
    NB_FDM(5) NB_FDM(6) NB_FDM(7) NB_FDM(8) NB_FDM(9) NB_FDM(10) NB_FDM(11) NB_FDM(12)
    NB_FDM(13) NB_FDM(14) NB_FDM(15) NB_FDM(16) NB_FDM(17) NB_FDM(18)
#undef NB_FDM
    default: return nullptr;
  }
}
template <typename T>
FdmFn<T> fdm_fixed(int nl) {
  return g_fixed_kernels ? fdm_fixed_any<T>(nl) : nullptr;
}

template <typename T>
size_t fdm_smem(int nl) {
  return sizeof(T) * (4 * size_t(nl) * nl * nl + 6 * nl * nl);
}
// shared bytes and threads of the fixed kernel for nl (0 when none)
template <typename T>
void fdm_fixed_shape(int nl, size_t *smem, int *threads) {
  switch (nl) {
#define NB_FDM(N)                              \
  case N:                                      \
    *smem = FdmShape<T, N>::SMEM;              \
    *threads = FdmShape<T, N>::THREADS;        \
    return;
    NB_FDM(5) NB_FDM(6) NB_FDM(7) NB_FDM(8) NB_FDM(9) NB_FDM(10) NB_FDM(11) NB_FDM(12)
    NB_FDM(13) NB_FDM(14) NB_FDM(15) NB_FDM(16) NB_FDM(17) NB_FDM(18)
#undef NB_FDM
    default: *smem = 0, *threads = 0;
  }
}
template <typename T>
size_t fdm_fixed_smem(int nl) {
  size_t sm;
  int th;
  fdm_fixed_shape<T>(nl, &sm, &th);
  return sm;
}

// FDM launch: the fixed-size kernel where one exists, else the general one
// (shared-memory limits raised once in the set-up)
template <typename T>
int launch_fdm(T *B, T *A, const T *s, const T *d, int nl, int nelt, cudaStream_t st) {
  if (FdmFn<T> fn = fdm_fixed<T>(nl)) {
    size_t sm;
    int th;
    fdm_fixed_shape<T>(nl, &sm, &th);
    fn<<<nelt, th, sm, st>>>(B, A, s, d);
  }
  else k_fdm<T><<<nelt, 256, fdm_smem<T>(nl), st>>>(B, A, s, d, nl);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

// extrude(B,0,1,A,0,-1), extrude(B,2,1,B,0,1), toreg3d (hsmg.f:1086-1090):
// each regular point adds, in the reference's face order, the neighbour
// contributions (gs'd ghost minus saved ghost) of the ghost faces whose
// layer-2 partner it is.
template <typename T>
__global__ void k_overlap_toreg(T *e_out, const T *B, const T *A, int nh, int nelt) {
  const int nl = nh + 2, nl2 = nl * nl, nh2 = nh * nh, lines = nh2 * nelt;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < lines; t += gridDim.x * blockDim.x) {
    const int e = t / nh2, ab = t - e * nh2, a = ab % nh + 1, b = ab / nh + 1;
    const int base = e * nl2 * nl;
    auto at = [&](int x, int y, int z) { return base + x + nl * y + nl2 * z; };
    T *eo = e_out + e * nh2 * nh + ab;
    for (int c0 = 1; c0 <= nh; c0 += kChunk) {
      T v[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u) {
        const int c = c0 + u;
        if (c > nh) break;
        T x = B[at(a, b, c)];
        if (a == 2) { const int g = at(0, b, c); x = add_rn(x, fma_rn(T(-1), A[g], B[g])); }
        if (a == nl - 3) { const int g = at(nl - 1, b, c); x = add_rn(x, fma_rn(T(-1), A[g], B[g])); }
        if (b == 2) { const int g = at(a, 0, c); x = add_rn(x, fma_rn(T(-1), A[g], B[g])); }
        if (b == nl - 3) { const int g = at(a, nl - 1, c); x = add_rn(x, fma_rn(T(-1), A[g], B[g])); }
        if (c == 2) { const int g = at(a, b, 0); x = add_rn(x, fma_rn(T(-1), A[g], B[g])); }
        if (c == nl - 3) { const int g = at(a, b, nl - 1); x = add_rn(x, fma_rn(T(-1), A[g], B[g])); }
        v[u] = x;
      }
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
        if (c0 + u <= nh) eo[(c0 + u - 1) * nh2] = v[u];
    }
  }
}

// Layer slots of coordinate x in an n-point line: bit s set when x sits in
// slot s of L = {0, 1, n-2, n-1}.
__device__ __forceinline__ int wt_slots(int x, int n) {
  return (x == 0) | (x == 1) << 1 | (x == n - 2) << 2 | (x == n - 1) << 3;
}
// h1mg_schwarz_wt3d2 (hsmg.f:1144-1178) at point (i, j, k) of an element:
// x *= sqrt(wt) over three sweeps of the layers L: x faces, then y faces of
// the x-interior, then z faces of the x- and y-interior.  A point takes the
// factor of every slot it sits in, in slot order (two slots coincide when
// n < 4).  we: the element's 12 n^2 weights, square-rooted at set-up.
template <typename T>
__device__ __forceinline__ T schwarz_weigh(T x, const T *we, int n, int i, int j, int k) {
  const int n2 = n * n, mi = wt_slots(i, n), mj = wt_slots(j, n);
  const T *w;
  int m;
  if (mi) w = we + j + n * k, m = mi;
  else if (mj) w = we + 4 * n2 + i + n * k, m = mj;
  else if ((m = wt_slots(k, n))) w = we + 8 * n2 + i + n * j;
  else return x;
#pragma unroll
  for (int sl = 0; sl < 4; ++sl)
    if (m >> sl & 1) x = mul_rn(x, w[sl * n2]);
  return x;
}

// h1mg_rstr (hsmg.f:1340-1360): do_wt (hsmg.f:1362-1391) then
// v = [J^T (x) J^T (x) J^T] u per element
template <typename T>
__global__ void k_rstr(T *v, const T *u, const T *wt, int nu, int nv, const T *jht,
                       const T *jh) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  const int nu3 = nu * nu * nu, nmax = max(nu, nv), nmax3 = nmax * nmax * nmax;
  T *us = sm, *vs = us + nmax3, *work = vs + nmax3, *work2 = work + nmax3,
    *Jt = work2 + nmax3, *J = Jt + nu * nv;
  const long e = blockIdx.x;
  const T *we = wt + e * 6L * nu * nu;
  for (int q = threadIdx.x; q < nu3; q += blockDim.x) {
    const int i = q % nu, j = (q / nu) % nu, k = q / (nu * nu);
    T x = u[e * nu3 + q];
    if (i == 0) x = mul_rn(x, we[j + nu * k + 0]);
    else if (i == nu - 1) x = mul_rn(x, we[j + nu * k + nu * nu]);
    else if (j == 0) x = mul_rn(x, we[i + nu * k + 2 * nu * nu]);
    else if (j == nu - 1) x = mul_rn(x, we[i + nu * k + 3 * nu * nu]);
    else if (k == 0) x = mul_rn(x, we[i + nu * j + 4 * nu * nu]);
    else if (k == nu - 1) x = mul_rn(x, we[i + nu * j + 5 * nu * nu]);
    us[q] = x;
  }
  load_shared(Jt, jht, nu * nv);
  load_shared(J, jh, nu * nv);
  __syncthreads();
  tensor3<T>(vs, us, nv, nu, Jt, J, J, work, work2);
  const int nv3 = nv * nv * nv;
  for (int q = threadIdx.x; q < nv3; q += blockDim.x) v[e * nv3 + q] = vs[q];
}

// h1mg_intp (hsmg.f:1436-1475) accumulated: out += [J (x) J (x) J] uc.
// With wt (the fine level's square-rooted Schwarz weights), out is first
// weighted as h1mg_schwarz_wt3d2 would have left it: the smoother's last
// pass, fused into the one kernel that reads its output next.
template <typename T>
__global__ void k_intp_add(T *out, const T *uc, int nu, int nv, const T *jh, const T *jht,
                           const T *wt) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  const int nmax = max(nu, nv), nmax3 = nmax * nmax * nmax;
  T *us = sm, *vs = us + nmax3, *work = vs + nmax3, *work2 = work + nmax3, *J = work2 + nmax3,
    *Jt = J + nu * nv;
  const long e = blockIdx.x;
  const int nu3 = nu * nu * nu, nv3 = nv * nv * nv;
  load_shared(us, uc + e * nu3, nu3);
  load_shared(J, jh, nu * nv);
  load_shared(Jt, jht, nu * nv);
  __syncthreads();
  tensor3<T>(vs, us, nv, nu, J, Jt, Jt, work, work2);
  const T *we = wt ? wt + e * 12 * nv * nv : nullptr;
  for (int q = threadIdx.x; q < nv3; q += blockDim.x) {
    T o = out[e * nv3 + q];
    if (we) o = schwarz_weigh(o, we, nv, q % nv, (q / nv) % nv, q / (nv * nv));
    out[e * nv3 + q] = add_rn(o, vs[q]);
  }
}

// Inter-level transfers with both sizes known at compile time: NU input
// and NV output points per direction.  tensor3_fx makes the sums of tensor3
// (same operands, same left-to-right order) with unrolled lines of G
// outputs each; the last pass hands every output to store(q, value).
template <typename T, int NV, int NU, int G, typename Store>
__device__ __forceinline__ void tensor3_fx(const T *u, const T *A, const T *Bt, const T *Ct,
                                           T *work, T *work2, Store store) {
  constexpr int NG = (NV + G - 1) / G;
  const int t = threadIdx.x, nt = blockDim.x;
  for (int it = t; it < NU * NU * NG; it += nt) {  // work(a, np) = sum_m A(a,m) u(m, np)
    const int np_ = it / NG, a0 = (it % NG) * G;
    T x[NU];
#pragma unroll
    for (int m = 0; m < NU; ++m) x[m] = u[m + np_ * NU];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int a = a0 + g < NV ? a0 + g : NV - 1;
      T acc = mul_rn(A[a], x[0]);
#pragma unroll
      for (int m = 1; m < NU; ++m) acc = fma_rn(A[a + m * NV], x[m], acc);
      if (a0 + g < NV) work[a + np_ * NV] = acc;
    }
  }
  __syncthreads();
  for (int it = t; it < NV * NU * NG; it += nt) {  // work2(a,b,p) = sum_n work(a,n,p) Bt(n,b)
    const int ap = it / NG, b0 = (it % NG) * G;
    const int a = ap % NV, p = ap / NV;
    const T *wp = work + NV * NU * p;
    T x[NU];
#pragma unroll
    for (int n = 0; n < NU; ++n) x[n] = wp[a + n * NV];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int b = b0 + g < NV ? b0 + g : NV - 1;
      T acc = mul_rn(x[0], Bt[b * NU]);
#pragma unroll
      for (int n = 1; n < NU; ++n) acc = fma_rn(x[n], Bt[n + b * NU], acc);
      if (b0 + g < NV) work2[a + NV * b + NV * NV * p] = acc;
    }
  }
  __syncthreads();
  for (int it = t; it < NV * NV * NG; it += nt) {  // v(ab, c) = sum_p work2(ab,p) Ct(p,c)
    const int ab = it / NG, c0 = (it % NG) * G;
    T x[NU];
#pragma unroll
    for (int p = 0; p < NU; ++p) x[p] = work2[ab + p * NV * NV];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int c = c0 + g < NV ? c0 + g : NV - 1;
      T acc = mul_rn(x[0], Ct[c * NU]);
#pragma unroll
      for (int p = 1; p < NU; ++p) acc = fma_rn(x[p], Ct[p + c * NU], acc);
      if (c0 + g < NV) store(ab + NV * NV * c, acc);
    }
  }
}

template <int NV>
constexpr int xfer_group() { return NV >= 8 ? 4 : 2; }

template <typename T, int NU, int NV>
constexpr size_t xfer_smem() {
  return sizeof(T) * (NU * NU * NU + NV * NU * NU + NV * NV * NU + 2 * NU * NV);
}

// k_rstr with NU (fine) -> NV (coarse) fixed
template <typename T, int NU, int NV>
__global__ void __launch_bounds__(256) k_rstr_fixed(T *v, const T *u, const T *wt,
                                                    const T *jht, const T *jh) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *us = reinterpret_cast<T *>(sm_raw), *work = us + NU * NU * NU, *work2 = work + NV * NU * NU,
    *Jt = work2 + NV * NV * NU, *J = Jt + NU * NV;
  constexpr int NU2 = NU * NU, NU3 = NU2 * NU, NV3 = NV * NV * NV;
  const int e = blockIdx.x;
  const T *we = wt + e * 6 * NU2;
  for (int q = threadIdx.x; q < NU3; q += blockDim.x) {
    const int i = q % NU, j = (q / NU) % NU, k = q / NU2;
    T x = u[e * NU3 + q];
    if (i == 0) x = mul_rn(x, we[j + NU * k + 0]);
    else if (i == NU - 1) x = mul_rn(x, we[j + NU * k + NU2]);
    else if (j == 0) x = mul_rn(x, we[i + NU * k + 2 * NU2]);
    else if (j == NU - 1) x = mul_rn(x, we[i + NU * k + 3 * NU2]);
    else if (k == 0) x = mul_rn(x, we[i + NU * j + 4 * NU2]);
    else if (k == NU - 1) x = mul_rn(x, we[i + NU * j + 5 * NU2]);
    us[q] = x;
  }
  load_shared(Jt, jht, NU * NV);
  load_shared(J, jh, NU * NV);
  __syncthreads();
  T *ve = v + e * NV3;
  tensor3_fx<T, NV, NU, xfer_group<NV>()>(us, Jt, J, J, work, work2,
                                          [&](int q, T val) { ve[q] = val; });
}

// k_intp_add with NU (coarse) -> NV (fine) fixed
template <typename T, int NU, int NV>
__global__ void __launch_bounds__(256) k_intp_fixed(T *out, const T *uc, const T *jh,
                                                    const T *jht, const T *wt) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *us = reinterpret_cast<T *>(sm_raw), *work = us + NU * NU * NU, *work2 = work + NV * NU * NU,
    *J = work2 + NV * NV * NU, *Jt = J + NU * NV;
  constexpr int NU3 = NU * NU * NU, NV3 = NV * NV * NV;
  const int e = blockIdx.x;
  load_shared(us, uc + e * NU3, NU3);
  load_shared(J, jh, NU * NV);
  load_shared(Jt, jht, NU * NV);
  __syncthreads();
  // the interpolant into shared memory, then one coalesced
  // read-modify-write of out
  T *vs = Jt + NU * NV;
  tensor3_fx<T, NV, NU, xfer_group<NV>()>(us, J, Jt, Jt, work, work2,
                                          [&](int q, T val) { vs[q] = val; });
  __syncthreads();
  T *oe = out + e * NV3;
  const T *we = wt ? wt + e * 12 * NV * NV : nullptr;
  for (int q = threadIdx.x; q < NV3; q += blockDim.x) {
    T o = oe[q];
    if (we) o = schwarz_weigh(o, we, NV, q % NV, (q / NV) % NV, q / (NV * NV));
    oe[q] = add_rn(o, vs[q]);
  }
}

// The fixed transfer kernels for a (fine, coarse) pair of level sizes:
// the pairs the default level choice makes for lx1 4..10 and the level
// lists of the deformed workloads; others take the general kernels.
template <typename T>
struct XferFixed {
  void (*rstr)(T *, const T *, const T *, const T *, const T *) = nullptr;
  void (*intp)(T *, const T *, const T *, const T *, const T *) = nullptr;
  size_t smem_rstr = 0, smem_intp = 0;
};
template <typename T>
XferFixed<T> xfer_fixed_any(int nf, int nc) {
  XferFixed<T> x;
#define NB_XF(F, C)                                              \
  if (nf == F && nc == C) {                                      \
    x.rstr = k_rstr_fixed<T, F, C>;                              \
    x.intp = k_intp_fixed<T, C, F>;                              \
    x.smem_rstr = xfer_smem<T, F, C>();                          \
    x.smem_intp = xfer_smem<T, C, F>() + sizeof(T) * F * F * F;  \
    return x;                                                    \
  }
  NB_XF(3, 2) NB_XF(4, 2) NB_XF(5, 3) NB_XF(6, 2) NB_XF(6, 3) NB_XF(6, 4) NB_XF(7, 4)
  NB_XF(8, 4) NB_XF(9, 4) NB_XF(10, 4) NB_XF(12, 6) NB_XF(16, 8)
#undef NB_XF
  return x;
}
template <typename T>
XferFixed<T> xfer_fixed(int nf, int nc) {
  return g_fixed_kernels ? xfer_fixed_any<T>(nf, nc) : XferFixed<T>();
}

// set-up helpers -------------------------------------------------------
__global__ void k_fill(double *a, double v, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = v;
}
// element faces = 1, rest 0 (h1mg_setup_rstr_wt, hsmg.f:211-229)
__global__ void k_faces_one(double *w, int n, int nelt) {
  const long n3 = long(n) * n * n, tot = n3 * nelt;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < tot;
       q += long(gridDim.x) * blockDim.x) {
    const int rr = int(q % n3);
    const int i = rr % n, j = (rr / n) % n, k = rr / (n * n);
    w[q] = (i == 0 || i == n - 1 || j == 0 || j == n - 1 || k == 0 || k == n - 1) ? 1.0 : 0.0;
  }
}
// wt(.,.,side,dir,e) = 1/w at the element faces (hsmg.f:233-247)
__global__ void k_rstr_wt(double *wt, const double *w, int n, int nelt) {
  const long n2 = long(n) * n, tot = n2 * nelt;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < tot;
       q += long(gridDim.x) * blockDim.x) {
    const long e = q / n2;
    const int a = int(q % n2) % n, b = int(q % n2) / n;
    const double *we = w + e * n2 * n;
    double *te = wt + e * 6 * n2;
    te[a + n * b + 0 * n2] = 1.0 / we[0 + n * a + n2 * b];
    te[a + n * b + 1 * n2] = 1.0 / we[(n - 1) + n * a + n2 * b];
    te[a + n * b + 2 * n2] = 1.0 / we[a + n * 0 + n2 * b];
    te[a + n * b + 3 * n2] = 1.0 / we[a + n * (n - 1) + n2 * b];
    te[a + n * b + 4 * n2] = 1.0 / we[a + n * b + n2 * 0];
    te[a + n * b + 5 * n2] = 1.0 / we[a + n * b + n2 * (n - 1)];
  }
}
// save ghost faces of B into A (setup version of the k_fdm side effect)
__global__ void k_save_ghost(double *A, const double *B, int nl, int nelt) {
  const long nl3 = long(nl) * nl * nl, tot = nl3 * nelt;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < tot;
       q += long(gridDim.x) * blockDim.x) {
    const int rr = int(q % nl3);
    if (ghost_face(rr % nl, (rr / nl) % nl, rr / (nl * nl), nl)) A[q] = B[q];
  }
}
// schwarz wt = 1/work at layers 1,2,n-1,n (h1mg_setup_schwarz_wt3d_2,
// hsmg.f:653-688)
__global__ void k_schwarz_wt_setup(double *wt, const double *w, int n, int nelt) {
  const long n2 = long(n) * n, tot = n2 * nelt;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < tot;
       q += long(gridDim.x) * blockDim.x) {
    const long e = q / n2;
    const int a = int(q % n2) % n, b = int(q % n2) / n;
    const double *we = w + e * n2 * n;
    double *te = wt + e * 12 * n2;
    const int L[4] = {0, 1, n - 2, n - 1};
    for (int s = 0; s < 4; ++s) {
      te[a + n * b + n2 * s + 0 * 4 * n2] = 1.0 / we[L[s] + n * a + n2 * b];
      te[a + n * b + n2 * s + 1 * 4 * n2] = 1.0 / we[a + n * L[s] + n2 * b];
      te[a + n * b + n2 * s + 2 * 4 * n2] = 1.0 / we[a + n * b + n2 * L[s]];
    }
  }
}

template <typename T>
__global__ void k_sqrt_inplace(T *a, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    a[q] = T(sqrt(a[q]));
}

size_t tensor_smem(int nmax, int extra) {
  return sizeof(double) * (4 * size_t(nmax) * nmax * nmax + extra);
}

int set_smem(const void *fn, size_t bytes) {
  NB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
  return NB_OK;
}

template <typename T>
int dmalloc(T **p, size_t n) {
  NB_CUDA(cudaMalloc(p, sizeof(T) * std::max<size_t>(n, 1)));
  return NB_OK;
}
template <typename T>
int upload(T **p, const std::vector<T> &h) {
  NB_TRY(dmalloc(p, h.size()));
  if (!h.empty())
    NB_CUDA(cudaMemcpy(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return NB_OK;
}

// h1mg_setup_fast1d_a / _b (hsmg.f:403-481); a, b are (n+3)^2 column-major
void fast1d_ab(double *a, double *b, int lbc, int rbc, double ll, double lm,
               double lr, const double *ah, const double *bh, int n) {
  const int na = n + 3;
  auto A = [&](int i, int j) -> double & { return a[i + j * na]; };
  auto Bm = [&](int i, int j) -> double & { return b[i + j * na]; };
  auto AH = [&](int i, int j) { return ah[i + j * (n + 1)]; };
  const int i0 = lbc == 1 ? 1 : 0, i1 = rbc == 1 ? n - 1 : n;
  for (int q = 0; q < na * na; ++q) a[q] = b[q] = 0.;
  double fac = 2.0 / lm;
  A(1, 1) = 1.0;
  A(n + 1, n + 1) = 1.0;
  for (int j = i0; j <= i1; ++j)
    for (int i = i0; i <= i1; ++i) A(i + 1, j + 1) = fac * AH(i, j);
  if (lbc == 0) {
    fac = 2.0 / ll;
    A(0, 0) = fac * AH(n - 1, n - 1);
    A(1, 0) = fac * AH(n, n - 1);
    A(0, 1) = fac * AH(n - 1, n);
    A(1, 1) = A(1, 1) + fac * AH(n, n);
  } else {
    A(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 2.0 / lr;
    A(n + 1, n + 1) = A(n + 1, n + 1) + fac * AH(0, 0);
    A(n + 2, n + 1) = fac * AH(1, 0);
    A(n + 1, n + 2) = fac * AH(0, 1);
    A(n + 2, n + 2) = fac * AH(1, 1);
  } else {
    A(n + 2, n + 2) = 1.0;
  }
  fac = 0.5 * lm;
  Bm(1, 1) = 1.0;
  Bm(n + 1, n + 1) = 1.0;
  for (int i = i0; i <= i1; ++i) Bm(i + 1, i + 1) = fac * bh[i];
  if (lbc == 0) {
    fac = 0.5 * ll;
    Bm(0, 0) = fac * bh[n - 1];
    Bm(1, 1) = Bm(1, 1) + fac * bh[n];
  } else {
    Bm(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 0.5 * lr;
    Bm(n + 1, n + 1) = Bm(n + 1, n + 1) + fac * bh[0];
    Bm(n + 2, n + 2) = fac * bh[1];
  } else {
    Bm(n + 2, n + 2) = 1.0;
  }
}

// h1mg_setup_fast1d (hsmg.f:380-401): s(nl,nl,2) and eigenvalues
int fast1d(double *s, double *lam, int nl, int lbc, int rbc, double ll,
           double lm, double lr, const double *ah, const double *bh, int n) {
  std::vector<double> b(nl * nl);
  fast1d_ab(s, b.data(), lbc, rbc, ll, lm, lr, ah, bh, n);
  const int info = generalev(s, b.data(), lam, nl);
  if (info) return fail(NB_ERR_NUMERIC, "h1mg setup: generalized eigensolve failed (%d)", info);
  auto rowz = [&](int e) {
    for (int j = 0; j < nl; ++j) s[(e - 1) + j * nl] = 0.;
  };
  if (lbc > 0) rowz(1);
  if (lbc == 1) rowz(2);
  if (rbc > 0) rowz(nl);
  if (rbc == 1) rowz(nl - 1);
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) s[nl * nl + i + j * nl] = s[j + i * nl];
  return NB_OK;
}

std::vector<int> level_mask(const Operator &op, int nh) {
  std::vector<int> list;
  const long n3 = long(nh) * nh * nh;
  for (int e = 0; e < op.nelt; ++e) {
    const unsigned f = op.face[e];
    if (!f) continue;
    for (int k = 0; k < nh; ++k)
      for (int j = 0; j < nh; ++j)
        for (int i = 0; i < nh; ++i) {
          const bool m = ((f & 1u) && i == 0) || ((f & 2u) && i == nh - 1) ||
                         ((f & 4u) && j == 0) || ((f & 8u) && j == nh - 1) ||
                         ((f & 16u) && k == 0) || ((f & 32u) && k == nh - 1);
          if (m) list.push_back(int(n3 * e + i + nh * j + nh * nh * k));
        }
  }
  return list;
}

GsHost numbering(const Operator &op, int nx) {
  const long n = long(nx) * nx * nx * op.nelt;
  std::vector<int64_t> glo(n);
  set_vert_box(glo.data(), nx, op.nelt, op.nelx, op.nely, op.lglel.data());
  GsHost h;
  gs_topology(glo.data(), int(n), &h);
  return h;
}

// the sum-overlap sequence of h1mg_schwarz_part1 (hsmg.f:1083-1090) from B
// (extended) into e (regular), with A as the ghost save area
int overlap_sum(const MgLevel &L, int nelt, double *e, double *B, double *A,
                cudaStream_t s) {
  k_save_ghost<<<grid_for(L.next), 256, 0, s>>>(A, B, L.nl, nelt);
  NB_TRY(gs_exec(L.gsx, B, 1, 1, 0, s));
  k_overlap_toreg<double><<<line_grid(L.nh, nelt), 256, 0, s>>>(e, B, A, L.nh, nelt);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

}  // namespace

__global__ void k_to_f32(float *y, const double *x, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    y[q] = float(x[q]);
}

int copy_f32(float **dst, const double *src, long n, cudaStream_t s) {
  NB_TRY(dmalloc(dst, size_t(n)));
  k_to_f32<<<grid_for(n), 256, 0, s>>>(*dst, src, n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

int mg_setup(Multigrid *mg, const Operator &op, const int *orders, int nlev,
             cudaStream_t s, int precision) {
  if (precision != 64 && precision != 32)
    return fail(NB_ERR_ARG, "h1mg: precision %d not 64 or 32", precision);
  mg->op = &op;
  mg->precision = precision;
  const int nx1 = op.lx, nelt = op.nelt;
  int ord[8] = {0};
  if (!orders) {
    static const int mgn2[10] = {1, 2, 2, 2, 2, 3, 3, 5, 5, 5};
    if (nx1 > 10)
      return fail(NB_ERR_UNSUPPORTED,
                  "h1mg_setup: the reference level choice reads an undefined "
                  "variable for lx1 > 10 (hsmg.f:65); pass explicit orders");
    if (nx1 < 4) return fail(NB_ERR_UNSUPPORTED, "h1mg_setup: lx1=%d < 4", nx1);
    int lmax = nx1 == 4 ? 2 : 3;
    int m2 = mgn2[nx1 - 1];
    if (nx1 == 8) m2 = 3;
    m2 = std::min(3, m2);
    ord[1] = 1;
    ord[2] = m2;
    ord[3] = m2 + 1;
    ord[lmax] = nx1 - 1;
    nlev = lmax;
  } else {
    if (nlev < 2 || nlev > 7) return fail(NB_ERR_ARG, "h1mg_setup: nlev=%d", nlev);
    for (int l = 1; l <= nlev; ++l) ord[l] = orders[l - 1];
    if (ord[nlev] != nx1 - 1)
      return fail(NB_ERR_ARG, "h1mg_setup: finest order %d != lx1-1", ord[nlev]);
  }
  for (int l = 1; l <= nlev; ++l)
    if (ord[l] < 1 || ord[l] + 3 > kMaxNl)
      return fail(NB_ERR_UNSUPPORTED, "h1mg_setup: level order %d", ord[l]);
  mg->nlev = nlev;
  std::vector<std::vector<double>> ah(nlev + 1), bh(nlev + 1), zh(nlev + 1);
  int maxnl = 0;
  for (int l = 1; l <= nlev; ++l) {
    MgLevel &L = mg->lv[l];
    L.order = ord[l];
    L.nh = ord[l] + 1;
    L.nl = L.nh + 2;
    L.n = long(L.nh) * L.nh * L.nh * nelt;
    L.next = long(L.nl) * L.nl * L.nl * nelt;
    maxnl = std::max(maxnl, L.nl);
    const int nh = L.nh;
    ah[l].resize(nh * nh);
    bh[l].resize(nh);
    zh[l].resize(nh);
    std::vector<double> c(nh * nh), d(nh * nh);
    semhat(ah[l].data(), bh[l].data(), c.data(), d.data(), zh[l].data(), ord[l]);
    if (op.brick && setup_on_device()) {
      // box numberings of nh and nh+2 points per direction (set_vert_box
      // through proxy_setupds, hsmg.f:161-166), built on the device
      NB_TRY(box_gs_device(nh, op.nelx, op.nely, op.nelz, &L.gs, s));
      NB_TRY(box_gs_device(nh + 2, op.nelx, op.nely, op.nelz, &L.gsx, s));
    } else {
      L.gs_host = numbering(op, nh);
      L.gsx_host = numbering(op, nh + 2);
      NB_TRY(gs_upload(L.gs_host, int(L.n), &L.gs, s));
      NB_TRY(gs_upload(L.gsx_host, int(L.next), &L.gsx, s));
    }
    NB_TRY(dmalloc(&L.e, L.n));
    NB_TRY(dmalloc(&L.r, L.n));
    const std::vector<int> mk = level_mask(op, nh);
    L.nmask = int(mk.size());
    NB_TRY(upload(&L.mask, mk));
  }
  // interpolation (h1mg_setup_intp / _intpm, hsmg.f:120-152)
  for (int l = 1; l < nlev; ++l) {
    const int nf = mg->lv[l + 1].nh, nc = mg->lv[l].nh;
    std::vector<double> jh(nf * nc), jht(nf * nc), w(2 * nc + 2);
    for (int i = 0; i < nf; ++i) {
      fd_weights_full(zh[l + 1][i], zh[l].data(), nc - 1, 1, w.data());
      for (int j = 0; j < nc; ++j) jh[i + j * nf] = w[j];
    }
    for (int j = 0; j < nc; ++j)
      for (int i = 0; i < nf; ++i) jht[j + i * nc] = jh[i + j * nf];
    NB_TRY(upload(&mg->lv[l].jh, jh));
    NB_TRY(upload(&mg->lv[l].jht, jht));
  }
  const long maxext = long(maxnl) * maxnl * maxnl * nelt;
  NB_TRY(dmalloc(&mg->A, maxext));
  NB_TRY(dmalloc(&mg->B, maxext));
  NB_TRY(dmalloc(&mg->w, op.n));
  // work arrays of the second stream's smoothers (levels 2..nlev-1)
  long lowext = 0;
  for (int l = 2; l < nlev; ++l)
    lowext = std::max(lowext, long(mg->lv[l].nh + 2) * (mg->lv[l].nh + 2) *
                                  (mg->lv[l].nh + 2) * nelt);
  if (lowext > 0 && precision == 64) {
    NB_TRY(dmalloc(&mg->A2, lowext));
    NB_TRY(dmalloc(&mg->B2, lowext));
  }
  if (!mg->s2) {
    NB_CUDA(cudaStreamCreateWithFlags(&mg->s2, cudaStreamNonBlocking));
    NB_CUDA(cudaEventCreateWithFlags(&mg->ev_fork, cudaEventDisableTiming));
    NB_CUDA(cudaEventCreateWithFlags(&mg->ev_join, cudaEventDisableTiming));
  }
  // restriction weights
  for (int l = 1; l <= nlev; ++l) {
    MgLevel &L = mg->lv[l];
    NB_TRY(dmalloc(&L.rstr_wt, size_t(L.nh) * L.nh * 6 * nelt));
    k_faces_one<<<grid_for(L.n), 256, 0, s>>>(mg->A, L.nh, nelt);
    NB_TRY(gs_exec(L.gs, mg->A, 1, 1, 0, s));
    k_rstr_wt<<<grid_for(long(L.nh) * L.nh * nelt), 256, 0, s>>>(L.rstr_wt, mg->A, L.nh, nelt);
    NB_CUDA(cudaGetLastError());
  }
  // FDM (h1mg_setup_fdm / _fast, hsmg.f:251-378): element lengths through a
  // dssum of face-centre markers on the finest numbering
  {
    const int lx = nx1;
    const long nxyz = long(lx) * lx * lx;
    std::vector<double> lw(op.n, 0.0);
    const double lm = 2.0;
    auto at = [&](int i, int j, int k, int e) -> double & {
      return lw[(i - 1) + lx * (j - 1) + long(lx) * lx * (k - 1) + nxyz * e];
    };
    for (int e = 0; e < nelt; ++e) {
      at(1, 2, 2, e) = lm;
      at(lx, 2, 2, e) = lm;
      at(2, 1, 2, e) = lm;
      at(2, lx, 2, e) = lm;
      at(2, 2, 1, e) = lm;
      at(2, 2, lx, e) = lm;
    }
    {  // dssum on the device maps (jl's sum order, bitwise the host's)
      double *d = nullptr;
      NB_CUDA(cudaMalloc(&d, op.n * sizeof(double)));
      int st = NB_OK;
      if (cudaMemcpyAsync(d, lw.data(), op.n * sizeof(double), cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
        st = fail(NB_ERR_CUDA, "h1mg_setup: lengths upload");
      if (!st) st = gs_exec(op.gs, d, 1, 1, 0, s);
      if (!st && (cudaMemcpyAsync(lw.data(), d, op.n * sizeof(double), cudaMemcpyDeviceToHost,
                                  s) != cudaSuccess ||
                  cudaStreamSynchronize(s) != cudaSuccess))
        st = fail(NB_ERR_CUDA, "h1mg_setup: lengths download");
      cudaFree(d);
      NB_TRY(st);
    }
    for (int l = 2; l <= nlev; ++l) {
      MgLevel &L = mg->lv[l];
      const int nl = L.nl, n = L.order;
      std::vector<double> S(size_t(nl) * nl * 6 * nelt), Dd(size_t(nl) * nl * nl * nelt);
      std::vector<double> lr(nl), ls(nl), lt(nl);
      // the 1-D problems depend only on the boundary flags and the three
      // lengths: each distinct one is solved once (bit-identical reuse)
      typedef std::tuple<int, int, uint64_t, uint64_t, uint64_t> Key;
      std::map<Key, std::pair<std::vector<double>, std::vector<double>>> memo;
      auto bits = [](double v) {
        uint64_t u;
        std::memcpy(&u, &v, sizeof(u));
        return u;
      };
      auto fast1d_once = [&](double *s1, double *lam, int lbc, int rbc, double ll,
                             double lrr_) -> int {
        const Key key(lbc, rbc, bits(ll), bits(lm), bits(lrr_));
        auto it = memo.find(key);
        if (it == memo.end()) {
          std::vector<double> sv(size_t(2) * nl * nl), lv(nl);
          NB_TRY(fast1d(sv.data(), lv.data(), nl, lbc, rbc, ll, lm, lrr_, ah[l].data(),
                        bh[l].data(), n));
          it = memo.emplace(key, std::make_pair(std::move(sv), std::move(lv))).first;
        }
        std::copy(it->second.first.begin(), it->second.first.end(), s1);
        std::copy(it->second.second.begin(), it->second.second.end(), lam);
        return NB_OK;
      };
      for (int e = 0; e < nelt; ++e) {
        const double llr = at(1, 2, 2, e) - lm, lrr = at(lx, 2, 2, e) - lm;
        const double lls = at(2, 1, 2, e) - lm, lrs = at(2, lx, 2, e) - lm;
        const double llt = at(2, 2, 1, e) - lm, lrt = at(2, 2, lx, e) - lm;
        const unsigned f = op.face[e];
        double *se = S.data() + size_t(nl) * nl * 6 * e;
        NB_TRY(fast1d_once(se, lr.data(), f & 1u ? 1 : 0, f & 2u ? 1 : 0, llr, lrr));
        NB_TRY(fast1d_once(se + 2 * nl * nl, ls.data(), f & 4u ? 1 : 0, f & 8u ? 1 : 0, lls,
                           lrs));
        NB_TRY(fast1d_once(se + 4 * nl * nl, lt.data(), f & 16u ? 1 : 0, f & 32u ? 1 : 0,
                           llt, lrt));
        auto vmax = [&](const std::vector<double> &v) {
          double t = -99.0e20;
          for (int q = 1; q <= nl - 2; ++q) t = std::max(t, v[q]);
          return t;
        };
        const double eps = 1.e-5 * (vmax(lr) + vmax(ls) + vmax(lt));
        double *de = Dd.data() + size_t(nl) * nl * nl * e;
        int il = 0;
        for (int k = 0; k < nl; ++k)
          for (int j = 0; j < nl; ++j)
            for (int i = 0; i < nl; ++i) {
              const double diag = lr[i] + ls[j] + lt[k];
              de[il++] = diag > eps ? 1.0 / diag : 0.0;
            }
      }
      NB_TRY(upload(&L.fast_s, S));
      NB_TRY(upload(&L.fast_d, Dd));
    }
  }
  // Schwarz weights (h1mg_setup_schwarz_wt3d_1, hsmg.f:572-622)
  for (int l = 2; l <= nlev; ++l) {
    MgLevel &L = mg->lv[l];
    NB_TRY(dmalloc(&L.schwarz_wt, size_t(L.nh) * L.nh * 12 * nelt));
    k_fill<<<grid_for(L.next), 256, 0, s>>>(mg->B, 1.0, L.next);
    NB_TRY(overlap_sum(L, nelt, L.e, mg->B, mg->A, s));
    NB_TRY(gs_exec(L.gs, L.e, 1, 1, 0, s));
    k_schwarz_wt_setup<<<grid_for(long(L.nh) * L.nh * nelt), 256, 0, s>>>(L.schwarz_wt, L.e,
                                                                        L.nh, nelt);
    NB_CUDA(cudaGetLastError());
  }
  const size_t sm_fdm = sizeof(double) * (4 * size_t(maxnl) * maxnl * maxnl + 6 * maxnl * maxnl);
  if (sm_fdm > 227 * 1024)
    return fail(NB_ERR_UNSUPPORTED, "h1mg: extended element of %d points too large", maxnl);
  NB_TRY(set_smem((const void *)k_fdm<double>, sm_fdm));
  NB_TRY(set_smem((const void *)k_rstr<double>, tensor_smem(maxnl, 2 * maxnl * maxnl)));
  NB_TRY(set_smem((const void *)k_intp_add<double>, tensor_smem(maxnl, 2 * maxnl * maxnl)));
  NB_TRY(set_smem((const void *)k_fdm<float>, sm_fdm / 2));
  NB_TRY(set_smem((const void *)k_rstr<float>, tensor_smem(maxnl, 2 * maxnl * maxnl) / 2));
  NB_TRY(set_smem((const void *)k_intp_add<float>, tensor_smem(maxnl, 2 * maxnl * maxnl) / 2));
  for (int l = 2; l <= nlev; ++l) {
    const int nl = mg->lv[l].nl;
    // the whole unified L1 as shared memory: occupancy is shared-memory bound
    if (FdmFn<double> fn = fdm_fixed_any<double>(nl)) {
      NB_TRY(set_smem((const void *)fn, fdm_fixed_smem<double>(nl)));
      NB_CUDA(cudaFuncSetAttribute((const void *)fn,
                                   cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    }
    if (FdmFn<float> fn = fdm_fixed_any<float>(nl)) {
      NB_TRY(set_smem((const void *)fn, fdm_fixed_smem<float>(nl)));
      NB_CUDA(cudaFuncSetAttribute((const void *)fn,
                                   cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    }
  }
  for (int l = 1; l < nlev; ++l) {
    const int nf = mg->lv[l + 1].nh, nc = mg->lv[l].nh;
    const XferFixed<double> xd = xfer_fixed_any<double>(nf, nc);
    const XferFixed<float> xf = xfer_fixed_any<float>(nf, nc);
    if (xd.rstr) {
      NB_TRY(set_smem((const void *)xd.rstr, xd.smem_rstr));
      NB_TRY(set_smem((const void *)xd.intp, xd.smem_intp));
      NB_TRY(set_smem((const void *)xf.rstr, xf.smem_rstr));
      NB_TRY(set_smem((const void *)xf.intp, xf.smem_intp));
    }
  }
  if (precision == 32) {
    for (int l = 1; l <= nlev; ++l) {
      MgLevel &L = mg->lv[l];
      NB_TRY(copy_f32(&L.rstr_wt_f, L.rstr_wt, long(L.nh) * L.nh * 6 * nelt, s));
      if (l >= 2) {
        NB_TRY(copy_f32(&L.fast_s_f, L.fast_s, long(L.nl) * L.nl * 6 * nelt, s));
        NB_TRY(copy_f32(&L.fast_d_f, L.fast_d, long(L.nl) * L.nl * L.nl * nelt, s));
        NB_TRY(copy_f32(&L.schwarz_wt_f, L.schwarz_wt, long(L.nh) * L.nh * 12 * nelt, s));
      }
      if (l < nlev) {
        const long nfc = long(mg->lv[l + 1].nh) * L.nh;
        NB_TRY(copy_f32(&L.jh_f, L.jh, nfc, s));
        NB_TRY(copy_f32(&L.jht_f, L.jht, nfc, s));
      }
      NB_TRY(dmalloc(&L.e_f, L.n));
      NB_TRY(dmalloc(&L.r_f, L.n));
    }
    NB_TRY(dmalloc(&mg->A_f, maxext));
    NB_TRY(dmalloc(&mg->B_f, maxext));
    NB_TRY(dmalloc(&mg->z_f, op.n));
    if (lowext > 0) {
      NB_TRY(dmalloc(&mg->A2_f, lowext));
      NB_TRY(dmalloc(&mg->B2_f, lowext));
    }
  }
  // the smoother applies sqrt(wt): taken once here, in the working precision
  for (int l = 2; l <= nlev; ++l) {
    MgLevel &L = mg->lv[l];
    const long nw = long(L.nh) * L.nh * 12 * nelt;
    k_sqrt_inplace<double><<<grid_for(nw), 256, 0, s>>>(L.schwarz_wt, nw);
    if (L.schwarz_wt_f) k_sqrt_inplace<float><<<grid_for(nw), 256, 0, s>>>(L.schwarz_wt_f, nw);
    NB_CUDA(cudaGetLastError());
  }
  NB_CUDA(cudaStreamSynchronize(s));
  return NB_OK;
}

namespace {

// Per-precision views of the level data.
template <typename T>
struct LevelView;
template <>
struct LevelView<double> {
  static const double *rstr_wt(const MgLevel &L) { return L.rstr_wt; }
  static const double *fast_s(const MgLevel &L) { return L.fast_s; }
  static const double *fast_d(const MgLevel &L) { return L.fast_d; }
  static const double *schwarz_wt(const MgLevel &L) { return L.schwarz_wt; }
  static const double *jh(const MgLevel &L) { return L.jh; }
  static const double *jht(const MgLevel &L) { return L.jht; }
  static double *e(MgLevel &L) { return L.e; }
  static double *r(MgLevel &L) { return L.r; }
  static double *A(Multigrid &m) { return m.A; }
  static double *B(Multigrid &m) { return m.B; }
  static double *A2(Multigrid &m) { return m.A2; }
  static double *B2(Multigrid &m) { return m.B2; }
  static constexpr int dom = 1;
};
template <>
struct LevelView<float> {
  static const float *rstr_wt(const MgLevel &L) { return L.rstr_wt_f; }
  static const float *fast_s(const MgLevel &L) { return L.fast_s_f; }
  static const float *fast_d(const MgLevel &L) { return L.fast_d_f; }
  static const float *schwarz_wt(const MgLevel &L) { return L.schwarz_wt_f; }
  static const float *jh(const MgLevel &L) { return L.jh_f; }
  static const float *jht(const MgLevel &L) { return L.jht_f; }
  static float *e(MgLevel &L) { return L.e_f; }
  static float *r(MgLevel &L) { return L.r_f; }
  static float *A(Multigrid &m) { return m.A_f; }
  static float *B(Multigrid &m) { return m.B_f; }
  static float *A2(Multigrid &m) { return m.A2_f; }
  static float *B2(Multigrid &m) { return m.B2_f; }
  static constexpr int dom = 2;
};

// h1mg_schwarz (hsmg.f:1036-1051) at level l: e = part1(r), masked; masks
// r first when mask_r (the finest level's r is masked by the caller).  The
// final e *= sqrt(W) (h1mg_schwarz_wt) is left to the interpolation that
// next reads e (mg_intp_add with weigh), which applies it on its load.
// A, B: extended work arrays of the stream s.
template <typename T>
int mg_schwarz(Multigrid &mg, T *e, T *r, int l, T *A, T *B, bool mask_r, cudaStream_t s) {
  typedef LevelView<T> V;
  MgLevel &L = mg.lv[l];
  const int nelt = mg.op->nelt;
  if (mask_r) NB_TRY(vec_mask<T>(r, L.mask, L.nmask, s));
  k_toext<T><<<line_grid(L.nl, nelt), 256, 0, s>>>(A, r, L.nh, nelt);
  NB_TRY(gs_exec(L.gsx, A, V::dom, 1, 0, s));
  NB_TRY(launch_fdm<T>(B, A, V::fast_s(L), V::fast_d(L), L.nl, nelt, s));
  NB_TRY(gs_exec(L.gsx, B, V::dom, 1, 0, s));
  k_overlap_toreg<T><<<line_grid(L.nh, nelt), 256, 0, s>>>(e, B, A, L.nh, nelt);
  NB_TRY(gs_exec(L.gs, e, V::dom, 1, 0, s));
  NB_TRY(vec_mask<T>(e, L.mask, L.nmask, s));
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

template <typename T>
int mg_rstr(Multigrid &mg, T *rc, const T *rf, int l, bool dssum, cudaStream_t s) {
  typedef LevelView<T> V;
  const MgLevel &F = mg.lv[l + 1], &C = mg.lv[l];
  const XferFixed<T> fx = xfer_fixed<T>(F.nh, C.nh);
  if (fx.rstr) {
    fx.rstr<<<mg.op->nelt, 256, fx.smem_rstr, s>>>(rc, rf, V::rstr_wt(F), V::jht(C), V::jh(C));
  } else {
    const int nmax = std::max(F.nh, C.nh);
    k_rstr<T><<<mg.op->nelt, 256, tensor_smem(nmax, 2 * F.nh * C.nh) * sizeof(T) / 8, s>>>(
        rc, rf, V::rstr_wt(F), F.nh, C.nh, V::jht(C), V::jh(C));
  }
  NB_CUDA(cudaGetLastError());
  if (dssum) NB_TRY(gs_exec(C.gs, rc, V::dom, 1, 0, s));
  return NB_OK;
}

// of += J ec from level l to l+1; weigh: first apply level l+1's Schwarz
// weights to of (the smoother's output there)
template <typename T>
int mg_intp_add(Multigrid &mg, T *of, const T *ec, int l, bool weigh, cudaStream_t s) {
  typedef LevelView<T> V;
  const MgLevel &F = mg.lv[l + 1], &C = mg.lv[l];
  const T *wt = weigh ? V::schwarz_wt(F) : nullptr;
  const XferFixed<T> fx = xfer_fixed<T>(F.nh, C.nh);
  if (fx.intp) {
    fx.intp<<<mg.op->nelt, 256, fx.smem_intp, s>>>(of, ec, V::jh(C), V::jht(C), wt);
  } else {
    const int nmax = std::max(F.nh, C.nh);
    k_intp_add<T><<<mg.op->nelt, 256, tensor_smem(nmax, 2 * F.nh * C.nh) * sizeof(T) / 8, s>>>(
        of, ec, C.nh, F.nh, V::jh(C), V::jht(C), wt);
  }
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

__global__ void k_to_f64(double *y, const float *x, long n) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += long(gridDim.x) * blockDim.x)
    y[q] = double(x[q]);
}

// ---- exact coarse solve ----------------------------------------------------
// b(i) = assembled residual at coarse vertex i (its first copy after dssum)
__global__ void k_coarse_gather(double *b, const double *e1, const int *prim, int nc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nc) b[i] = e1[prim[i]];
}
// e1(q) = x(gid(q)), 0 at masked points
__global__ void k_coarse_scatter(double *e1, const double *x, const int *gid, long n1) {
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n1;
       q += long(gridDim.x) * blockDim.x) {
    const int c = gid[q];
    e1[q] = c >= 0 ? x[c] : 0.0;
  }
}
// y = A x for the dense inverse: one warp per row, lane-strided partial
// sums in a fixed order, then a fixed shuffle tree
__global__ void __launch_bounds__(256) k_dense_mv(double *y, const double *A,
                                                  const double *x, int n) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double *row = A + size_t(warp) * n;
  double acc = 0.0;
  for (int j = lane; j < n; j += 32) acc = fma_rn(row[j], x[j], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[warp] = acc;
}

int coarse_apply(Multigrid &mg, cudaStream_t s) {
  MgLevel &C = mg.lv[1];
  k_coarse_gather<<<(mg.nc + 255) / 256, 256, 0, s>>>(mg.c_b, C.e, mg.c_prim, mg.nc);
  k_dense_mv<<<(mg.nc * 32 + 255) / 256, 256, 0, s>>>(mg.c_x, mg.c_ainv, mg.c_b, mg.nc);
  k_coarse_scatter<<<grid_for(C.n), 256, 0, s>>>(C.e, mg.c_x, mg.c_gid, C.n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

// The V-cycle of h1mg_solve (hsmg.f:960-1034) in precision T from level Lm
// down; the coarse "solve" (copy + dssum + mask, hsmg.f:945-957) is always
// FP64.  rT is the top-level right-hand side, zT the result.
//
// The cycle is additive: every level's Schwarz step reads only its own
// restricted residual, and the corrections meet on the way up.  So after
// the finest r is masked, the finest smoother runs on s while the
// restrictions, the coarser smoothers, the coarse solve and the
// interpolations up to level Lm-1 run on the second stream s2 (with their
// own work arrays); s waits for them before the last interpolation.  Each
// kernel computes what it did in one stream.
template <typename T>
int vcycle(Multigrid &mg, T *zT, T *rT, cudaStream_t s) {
  typedef LevelView<T> V;
  const int Lm = mg.nlev;
  MgLevel &Top = mg.lv[Lm];
  NB_TRY(vec_mask<T>(rT, Top.mask, Top.nmask, s));
  T *rTop = V::r(Top);
  if (rTop != rT) NB_TRY(vec_copy<T>(rTop, rT, Top.n, s));
  NB_CUDA(cudaEventRecord(mg.ev_fork, s));
  NB_TRY(mg_schwarz<T>(mg, zT, rT, Lm, V::A(mg), V::B(mg), false, s));
  cudaStream_t s2 = mg.s2;
  NB_CUDA(cudaStreamWaitEvent(s2, mg.ev_fork, 0));
  for (int l = Lm - 1; l >= 2; --l) {
    NB_TRY(mg_rstr<T>(mg, V::r(mg.lv[l]), V::r(mg.lv[l + 1]), l, true, s2));
    NB_TRY(mg_schwarz<T>(mg, V::e(mg.lv[l]), V::r(mg.lv[l]), l, V::A2(mg), V::B2(mg), true,
                         s2));
  }
  MgLevel &C = mg.lv[1];
  NB_TRY(mg_rstr<T>(mg, V::r(C), V::r(mg.lv[2]), 1, false, s2));
  if (std::is_same<T, double>::value) {
    NB_TRY(vec_mask<double>(C.r, C.mask, C.nmask, s2));
    NB_TRY(vec_copy<double>(C.e, C.r, C.n, s2));  // hsmg_coarse_solve
    NB_TRY(gs_exec(C.gs, C.e, 1, 1, 0, s2));
    if (mg.coarse_exact) NB_TRY(coarse_apply(mg, s2));
    NB_TRY(vec_mask<double>(C.e, C.mask, C.nmask, s2));
  } else {
    // FP64 coarse solve between the FP32 legs
    k_to_f64<<<grid_for(C.n), 256, 0, s2>>>(C.r, C.r_f, C.n);
    NB_TRY(vec_mask<double>(C.r, C.mask, C.nmask, s2));
    NB_TRY(vec_copy<double>(C.e, C.r, C.n, s2));
    NB_TRY(gs_exec(C.gs, C.e, 1, 1, 0, s2));
    if (mg.coarse_exact) NB_TRY(coarse_apply(mg, s2));
    NB_TRY(vec_mask<double>(C.e, C.mask, C.nmask, s2));
    k_to_f32<<<grid_for(C.n), 256, 0, s2>>>(C.e_f, C.e, C.n);
    NB_CUDA(cudaGetLastError());
  }
  for (int l = 2; l <= Lm - 1; ++l)
    NB_TRY(mg_intp_add<T>(mg, V::e(mg.lv[l]), V::e(mg.lv[l - 1]), l - 1, true, s2));
  NB_CUDA(cudaEventRecord(mg.ev_join, s2));
  NB_CUDA(cudaStreamWaitEvent(s, mg.ev_join, 0));
  return mg_intp_add<T>(mg, zT, V::e(mg.lv[Lm - 1]), Lm - 1, true, s);
}

}  // namespace

void mg_set_fixed_kernels(bool on) { g_fixed_kernels = on; }

// R A P of the V-cycle's transfers on a level-1 vector x1 (local copies):
// the result r1 is assembled (dssum) and masked, as the coarse step sees it.
static int coarse_rap(Multigrid &mg, const double *g, double *x1, double *z, double *w,
                      cudaStream_t s) {
  const Operator &op = *mg.op;
  const int L = mg.nlev;
  // P: e_2 = J e_1, ..., z = J e_{L-1} (the unwinding of h1mg_solve)
  const double *src = x1;
  for (int l = 2; l < L; ++l) {
    NB_CUDA(cudaMemsetAsync(mg.lv[l].e, 0, mg.lv[l].n * sizeof(double), s));
    NB_TRY(mg_intp_add<double>(mg, mg.lv[l].e, src, l - 1, false, s));
    src = mg.lv[l].e;
  }
  NB_CUDA(cudaMemsetAsync(z, 0, op.n * sizeof(double), s));
  NB_TRY(mg_intp_add<double>(mg, z, src, L - 1, false, s));
  // A
  metric_fx_invalidate(op);
  NB_TRY(apply_ax<double>(op, w, z, g, s));
  // R: the downward leg, masked at every level as h1mg_schwarz masks r
  MgLevel &Top = mg.lv[L];
  NB_TRY(vec_mask<double>(w, Top.mask, Top.nmask, s));
  NB_TRY(vec_copy<double>(Top.r, w, Top.n, s));
  for (int l = L - 1; l >= 2; --l) {
    NB_TRY(mg_rstr<double>(mg, mg.lv[l].r, mg.lv[l + 1].r, l, true, s));
    NB_TRY(vec_mask<double>(mg.lv[l].r, mg.lv[l].mask, mg.lv[l].nmask, s));
  }
  MgLevel &C = mg.lv[1];
  NB_TRY(mg_rstr<double>(mg, C.r, mg.lv[2].r, 1, false, s));
  NB_TRY(vec_mask<double>(C.r, C.mask, C.nmask, s));
  NB_TRY(gs_exec(C.gs, C.r, 1, 1, 0, s));
  return NB_OK;
}

int mg_setup_coarse(Multigrid *mg, const double *g, cudaStream_t s) {
  const Operator &op = *mg->op;
  MgLevel &C = mg->lv[1];
  if (C.nh != 2)
    return fail(NB_ERR_UNSUPPORTED, "exact coarse solve: the coarsest level must be order 1");
  if (!op.brick || op.mask_mode != 1)
    return fail(NB_ERR_UNSUPPORTED, "exact coarse solve: box meshes with the full mask only");
  const int nx = op.nelx, ny = op.nely, nz = op.nelz, nelt = op.nelt;
  const int vx = nx + 1, vy = ny + 1, vz = nz + 1;
  const long nv = long(vx) * vy * vz;
  // unmasked vertices, compressed in lexicographic order
  std::vector<int> cidx(nv, -1);
  std::vector<int> cv;  // coarse index -> vertex
  for (int k = 1; k < vz - 1; ++k)
    for (int j = 1; j < vy - 1; ++j)
      for (int i = 1; i < vx - 1; ++i) {
        const long v = i + long(vx) * (j + long(vy) * k);
        cidx[v] = int(cv.size());
        cv.push_back(int(v));
      }
  const int nc = int(cv.size());
  if (nc == 0) return fail(NB_ERR_UNSUPPORTED, "exact coarse solve: no interior vertex");
  if (nc > kMaxCoarse)
    return fail(NB_ERR_UNSUPPORTED, "exact coarse solve: %d coarse unknowns (at most %d)", nc,
                kMaxCoarse);
  const long n1 = C.n;  // 8 * nelt
  std::vector<int> gid(n1, -1), prim(nc, -1);
  std::vector<int> vert(n1);
  for (int e = 0; e < nelt; ++e) {
    const int ex = e % nx, ey = (e / nx) % ny, ez = e / (nx * ny);
    for (int q = 0; q < 8; ++q) {
      const int i = q & 1, j = (q >> 1) & 1, k = q >> 2;
      const long v = (ex + i) + long(vx) * ((ey + j) + long(vy) * (ez + k));
      const long lq = long(8) * e + q;
      vert[lq] = int(v);
      gid[lq] = cidx[v];
      if (cidx[v] >= 0 && prim[cidx[v]] < 0) prim[cidx[v]] = int(lq);
    }
  }
  double *x1 = nullptr, *z = nullptr, *w = nullptr;
  NB_CUDA(cudaMalloc(&x1, n1 * sizeof(double)));
  NB_CUDA(cudaMalloc(&z, op.n * sizeof(double)));
  NB_CUDA(cudaMalloc(&w, op.n * sizeof(double)));
  int st = NB_OK;
  // probes: 27 colourings, (vx mod 3, vy mod 3, vz mod 3)
  std::vector<double> A(size_t(nc) * nc, 0.0), hx(n1), hr(n1);
  for (int c = 0; c < 27 && !st; ++c) {
    const int cx = c % 3, cy = (c / 3) % 3, cz = c / 9;
    for (long q = 0; q < n1; ++q) {
      const int v = vert[q];
      const int ix = v % vx, iy = (v / vx) % vy, iz = v / (vx * vy);
      hx[q] = (gid[q] >= 0 && ix % 3 == cx && iy % 3 == cy && iz % 3 == cz) ? 1.0 : 0.0;
    }
    if (cudaMemcpy(x1, hx.data(), n1 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      st = fail(NB_ERR_CUDA, "exact coarse solve: upload");
    if (!st) st = coarse_rap(*mg, g, x1, z, w, s);
    if (!st && (cudaMemcpyAsync(hr.data(), C.r, n1 * sizeof(double), cudaMemcpyDeviceToHost,
                                s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess))
      st = fail(NB_ERR_CUDA, "exact coarse solve: probe");
    for (int i = 0; i < nc && !st; ++i) {
      const int v = cv[i];
      const int ix = v % vx, iy = (v / vx) % vy, iz = v / (vx * vy);
      // the one vertex of this colour within distance 1
      auto pick = [](int a, int col) {
        for (int d = -1; d <= 1; ++d)
          if (((a + d) % 3 + 3) % 3 == col) return a + d;
        return -1;
      };
      const int jx = pick(ix, cx), jy = pick(iy, cy), jz = pick(iz, cz);
      if (jx < 0 || jy < 0 || jz < 0 || jx >= vx || jy >= vy || jz >= vz) continue;
      const int cj = cidx[jx + long(vx) * (jy + long(vy) * jz)];
      if (cj < 0) continue;
      A[size_t(i) * nc + cj] = hr[prim[i]];
    }
  }
  // check: the probed matrix reproduces R A P on a random vector
  if (!st) {
    uint64_t z64 = 0x9E3779B97F4A7C15ull;
    std::vector<double> xc(nc);
    for (int i = 0; i < nc; ++i) {
      z64 ^= z64 << 13, z64 ^= z64 >> 7, z64 ^= z64 << 17;
      xc[i] = double(z64 >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
    for (long q = 0; q < n1; ++q) hx[q] = gid[q] >= 0 ? xc[gid[q]] : 0.0;
    if (cudaMemcpy(x1, hx.data(), n1 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      st = fail(NB_ERR_CUDA, "exact coarse solve: upload");
    if (!st) st = coarse_rap(*mg, g, x1, z, w, s);
    if (!st && (cudaMemcpyAsync(hr.data(), C.r, n1 * sizeof(double), cudaMemcpyDeviceToHost,
                                s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess))
      st = fail(NB_ERR_CUDA, "exact coarse solve: check");
    double emax = 0.0, ymax = 0.0, amax = 0.0, asym = 0.0;
    for (int i = 0; i < nc && !st; ++i) {
      double y = 0.0;
      for (int j = 0; j < nc; ++j) y += A[size_t(i) * nc + j] * xc[j];
      emax = std::max(emax, std::fabs(y - hr[prim[i]]));
      ymax = std::max(ymax, std::fabs(hr[prim[i]]));
    }
    for (int i = 0; i < nc && !st; ++i)
      for (int j = 0; j < i; ++j) {
        amax = std::max(amax, std::fabs(A[size_t(i) * nc + j]));
        asym = std::max(asym, std::fabs(A[size_t(i) * nc + j] - A[size_t(j) * nc + i]));
      }
    if (!st && emax > 1e-10 * ymax)
      st = fail(NB_ERR_NUMERIC, "exact coarse solve: probing mismatch %.3e", emax / ymax);
    if (!st && asym > 1e-10 * amax)
      st = fail(NB_ERR_NUMERIC, "exact coarse solve: R A P not symmetric (%.3e)", asym / amax);
  }
  cudaFree(x1);
  cudaFree(z);
  cudaFree(w);
  if (st) return st;
  // symmetrise, banded Cholesky, dense inverse (columns in parallel)
  int bw = 0;
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < i; ++j) {
      const double a = 0.5 * (A[size_t(i) * nc + j] + A[size_t(j) * nc + i]);
      A[size_t(i) * nc + j] = A[size_t(j) * nc + i] = a;
      if (a != 0.0) bw = std::max(bw, i - j);
    }
  std::vector<double> Lb(size_t(nc) * (bw + 1), 0.0);  // L(i, i-k) at [i*(bw+1)+k]
  auto Lat = [&](int i, int j) -> double & { return Lb[size_t(i) * (bw + 1) + (i - j)]; };
  for (int i = 0; i < nc; ++i)
    for (int j = std::max(0, i - bw); j <= i; ++j) {
      double sum = A[size_t(i) * nc + j];
      for (int k = std::max(std::max(0, i - bw), j - bw); k < j; ++k) sum -= Lat(i, k) * Lat(j, k);
      if (i == j) {
        if (!(sum > 0.0)) return fail(NB_ERR_NUMERIC, "exact coarse solve: not positive definite");
        Lat(i, i) = std::sqrt(sum);
      } else {
        Lat(i, j) = sum / Lat(j, j);
      }
    }
  std::vector<double> inv(size_t(nc) * nc);
  const int nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int t = 0; t < nth; ++t)
    th.emplace_back([&, t]() {
      std::vector<double> y(nc);
      for (int col = t; col < nc; col += nth) {
        // L y = e_col
        for (int i = 0; i < nc; ++i) {
          double sum = i == col ? 1.0 : 0.0;
          for (int k = std::max(0, i - bw); k < i; ++k) sum -= Lat(i, k) * y[k];
          y[i] = sum / Lat(i, i);
        }
        // L^T x = y
        for (int i = nc - 1; i >= 0; --i) {
          double sum = y[i];
          for (int k = i + 1; k <= std::min(nc - 1, i + bw); ++k) sum -= Lat(k, i) * y[k];
          y[i] = sum / Lat(i, i);
        }
        for (int i = 0; i < nc; ++i) inv[size_t(i) * nc + col] = y[i];
      }
    });
  for (auto &t : th) t.join();
  NB_TRY(upload(&mg->c_ainv, inv));
  NB_TRY(upload(&mg->c_gid, gid));
  NB_TRY(upload(&mg->c_prim, prim));
  NB_TRY(dmalloc(&mg->c_b, nc));
  NB_TRY(dmalloc(&mg->c_x, nc));
  mg->nc = nc;
  mg->coarse_exact = true;
  NB_CUDA(cudaStreamSynchronize(s));
  return NB_OK;
}

int mg_solve_f32(Multigrid &mg, cudaStream_t s) {
  if (mg.precision != 32) return fail(NB_ERR_STATE, "mg_solve_f32: FP32 smoother only");
  return vcycle<float>(mg, mg.z_f, mg.lv[mg.nlev].r_f, s);
}

int mg_solve(Multigrid &mg, double *z, double *rhs, cudaStream_t s) {
  if (mg.precision == 64) return vcycle<double>(mg, z, rhs, s);
  MgLevel &Top = mg.lv[mg.nlev];
  // the reference masks rhs in place (h1mg_schwarz_part1, hsmg.f:1067)
  NB_TRY(vec_mask<double>(rhs, Top.mask, Top.nmask, s));
  k_to_f32<<<grid_for(Top.n), 256, 0, s>>>(Top.r_f, rhs, Top.n);
  NB_CUDA(cudaGetLastError());
  NB_TRY(vcycle<float>(mg, mg.z_f, Top.r_f, s));
  k_to_f64<<<grid_for(Top.n), 256, 0, s>>>(z, mg.z_f, Top.n);
  NB_CUDA(cudaGetLastError());
  return NB_OK;
}

}  // namespace nb

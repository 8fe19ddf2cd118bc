// nb_internal.h -- shared declarations of the nekbone_gb300 native library.
//
// The library is the GB300 (sm_103a) implementation of Nekbone's spectral
// element Poisson CG hot path: the matrix-free operator ax (cg.f:96-212), the
// jl gather-scatter dssum/gs_op (prox_dssum.f:2-12, jl/gs.c:1029-1045), the CG
// vector kernels (math.f:534-617, cg.f:2-84) and the hsmg multigrid
// preconditioner (hsmg.f).  Host-side setup (GLL points, derivative matrices,
// global numbering, gather-scatter topology, multigrid set-up) is C++; every
// per-iteration operation is a CUDA kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace nb {

// ---------------------------------------------------------------- errors --
// Status codes returned by every entry point (0 = ok).
enum Status : int {
  NB_OK = 0,
  NB_ERR_ARG = 1,        // invalid argument (size, dom, op, nullptr ...)
  NB_ERR_HANDLE = 2,     // invalid or freed handle
  NB_ERR_CUDA = 3,       // a CUDA runtime call failed
  NB_ERR_STATE = 4,      // call made before the set-up it depends on
  NB_ERR_NUMERIC = 5,    // non-finite value or failed factorisation
  NB_ERR_UNSUPPORTED = 6 // size or mode outside what the kernels support
};

// Records an error.  In the reference error mode (the default) the message is
// printed and the process exits with status 1, as jl's fail() does
// (jl/fail.c:11-52); in the returning mode the status is stored and returned.
int fail(int status, const char *fmt, ...);
int last_status();
const char *last_message();
void clear_status();
int error_mode();
void set_error_mode(int mode);

#define NB_CUDA(call)                                                      \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess)                                                 \
      return ::nb::fail(::nb::NB_ERR_CUDA, "%s:%d %s: %s", __FILE__,       \
                        __LINE__, #call, cudaGetErrorString(e_));          \
  } while (0)

#define NB_TRY(expr)            \
  do {                          \
    int s_ = (expr);            \
    if (s_ != 0) return s_;     \
  } while (0)

// The device error word of bounded waits (allocated on first use) and its
// check, which synchronises the stream and fails if a wait ran out.
unsigned *device_error_word();
int device_error_check(cudaStream_t s);
// Whether launches enqueued now run the bulk-copy timeout self-test
// (nb_set_wait_test): their metric-copy waits run out on purpose.
int wait_test_mode();

constexpr int kMaxLx = 16;     // largest lx1 with a specialised ax kernel
constexpr int kMaxNl = 24;     // largest 1-D size of a multigrid tensor apply

// ------------------------------------------------------------ host setup --
// speclib.f / semhat.f restatements used by the product's own set-up.
void zwgll(double *z, double *w, int np);
void fd_weights_full(double xx, const double *x, int n, int m, double *c);
void semhat(double *a, double *b, double *c, double *d, double *z, int n);
void cubic(int *mx, int *my, int *mz, int np);
int mod1(int i, int n);
void get_exyz(int *ex, int *ey, int *ez, int eg, int nelx, int nely);
void set_vert_box(int64_t *glo_num, int nx, int nelt, int nelx, int nely,
                  const int *lglel);
// face bits of element ie (0-based) on the domain boundary, as get_face
// (cg.f:302-368) decides them: bit0 x=1, bit1 x=nx, bit2 y=1, bit3 y=nx,
// bit4 z=1, bit5 z=nx.
unsigned face_bits(int eg, int nelx, int nely, int nelz);
int generalev(double *a, double *b, double *lam, int n);

// ------------------------------------------------------- gather-scatter --
// Device form of a jl gather-scatter handle.  A group is a global id shared
// by several local indices; the first member is the primary.  Gather uses the
// "unflagged" member lists, scatter the "all" lists (gs.c:1041-1044).
struct GsDevice {
  int n = 0;                  // local vector length
  int ng = 0;                 // groups in the symmetric fast path
  int *off = nullptr;         // ng+1 offsets into idx
  int *idx = nullptr;         // members, primary first, jl order
  bool symmetric = true;      // no flagged ids: gather map == scatter map
  // general (flagged) path: separate maps
  int ng_g = 0, ng_s = 0, nfp = 0;
  int *off_g = nullptr, *idx_g = nullptr;
  int *off_s = nullptr, *idx_s = nullptr;
  int *fprim = nullptr;       // flagged primaries (init to the identity)
};

struct GsHost {
  std::vector<uint32_t> map[3]; // jl-format maps: unflagged, all, flagged prim.
};

// Builds the jl local topology of ids[0..n) (nonzero_ids gs.c:88-113 and
// local_map gs.c:330-357).
void gs_topology(const int64_t *ids, int n, GsHost *out);
int gs_upload(const GsHost &h, int n, GsDevice *d, cudaStream_t s);
void gs_release(GsDevice *d);
// u: device vector; dom 1 double, 2 float, 3 int, 4 int64; op 1..4.
int gs_exec(const GsDevice &d, void *u, int dom, int op, int transpose,
            cudaStream_t s);

}  // namespace nb

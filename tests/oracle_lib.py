"""ctypes binding of the CPU oracle (oracle/nb_oracle.c) -- the checker the
tests compare the CUDA path against.  Builds the oracle with make on first
use (gcc is available wherever the tests run)."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE = ROOT / "oracle"

_libs: dict[int, C.CDLL] = {}


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def load(fma: bool = True) -> C.CDLL:
    key = 1 if fma else 0
    if key in _libs:
        return _libs[key]
    name = "liboracle_fma.so" if fma else "liboracle.so"
    path = ORACLE / name
    src = ORACLE / "nb_oracle.c"
    if not path.exists() or path.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-C", str(ORACLE), name], check=True, capture_output=True)
    L = C.CDLL(str(path))
    L.orc_glsc3.restype = C.c_double
    L.orc_ctx_new.restype = C.c_void_p
    L.orc_gs_setup.restype = C.c_void_p
    L.orc_ctx_dxm1.restype = C.POINTER(C.c_double)
    L.orc_ctx_wxm1.restype = C.POINTER(C.c_double)
    L.orc_flop_a.restype = C.c_double
    L.orc_flop_cg.restype = C.c_double
    for f in ("orc_ctx_free", "orc_ctx_reset_mask", "orc_setup_g", "orc_set_multiplicity",
              "orc_set_f", "orc_dssum", "orc_maskit", "orc_ax", "orc_ax_local", "orc_ax_e",
              "orc_cg", "orc_h1mg_setup", "orc_h1mg_solve", "orc_h1mg_nlev", "orc_h1mg_order",
              "orc_h1mg_fdm_copy", "orc_ctx_n", "orc_flop_a", "orc_flop_cg",
              "orc_ctx_dxm1", "orc_ctx_wxm1", "orc_ctx_set_threads"):
        getattr(L, f).argtypes = None
    _libs[key] = L
    return L


def zwgll(np_: int, fma: bool = True):
    L = load(fma)
    z, w = np.zeros(np_), np.zeros(np_)
    L.orc_zwgll(_p(z), _p(w), C.c_int(np_))
    return z, w


def semhat(n: int, fma: bool = True):
    L = load(fma)
    m = n + 1
    a, c, d = np.zeros(m * m), np.zeros(m * m), np.zeros(m * m)
    b, z = np.zeros(m), np.zeros(m)
    L.orc_semhat(_p(a), _p(b), _p(c), _p(d), _p(z), C.c_int(n))
    return a, b, c, d, z


def cubic(np_: int):
    L = load()
    mx, my, mz = C.c_int(), C.c_int(), C.c_int()
    L.orc_cubic(C.byref(mx), C.byref(my), C.byref(mz), C.c_int(np_))
    return mx.value, my.value, mz.value


def set_vert_box(nx, nelt, nelx, nely, nelz, lglel):
    L = load()
    g = np.zeros(nx ** 3 * nelt, dtype=np.int64)
    lg = np.ascontiguousarray(lglel, dtype=np.int32)
    L.orc_set_vert_box(_p(g), C.c_int(nx), C.c_int(nelt), C.c_int(nelx), C.c_int(nely),
                       C.c_int(nelz), _p(lg))
    return g


def mxm(a, n1, b, n2, n3, fma=True):
    L = load(fma)
    c = np.zeros(n1 * n3)
    L.orc_mxm(_p(np.ascontiguousarray(a, dtype=np.float64)), C.c_int(n1),
              _p(np.ascontiguousarray(b, dtype=np.float64)), C.c_int(n2), _p(c), C.c_int(n3))
    return c


class Gs:
    """The oracle's restatement of a jl gather-scatter handle."""

    def __init__(self, ids, fma=True):
        self.L = load(fma)
        self.ids = np.ascontiguousarray(ids, dtype=np.int64)
        self.h = self.L.orc_gs_setup(_p(self.ids), C.c_int(len(self.ids)))

    def maps(self):
        out = []
        for w in range(3):
            n = self.L.orc_gs_map_len(C.c_void_p(self.h), C.c_int(w))
            m = np.zeros(n, dtype=np.uint32)
            self.L.orc_gs_map_copy(C.c_void_p(self.h), C.c_int(w), _p(m))
            out.append(m)
        return out

    def op(self, u, dom, op, transpose):
        self.L.orc_gs_op(C.c_void_p(self.h), _p(u), C.c_int(dom), C.c_int(op), C.c_int(transpose))

    def __del__(self):
        try:
            self.L.orc_gs_free(C.c_void_p(self.h))
        except Exception:
            pass


class Ctx:
    """The oracle's solver context (the reference's common blocks)."""

    def __init__(self, nelx, nely, nelz, nx1, mask_mode=0, lglel=None, nthreads=1, fma=True):
        self.L = load(fma)
        self.nelx, self.nely, self.nelz, self.nx1 = nelx, nely, nelz, nx1
        self.nelt = nelx * nely * nelz
        self.n = self.nelt * nx1 ** 3
        self.lglel = (np.arange(1, self.nelt + 1, dtype=np.int32) if lglel is None
                      else np.ascontiguousarray(lglel, dtype=np.int32))
        self.h = self.L.orc_ctx_new(C.c_int(nelx), C.c_int(nely), C.c_int(nelz),
                                    C.c_int(self.nelt), C.c_int(nx1), _p(self.lglel),
                                    C.c_int(mask_mode), C.c_int(nthreads))

    @property
    def hv(self):
        return C.c_void_p(self.h)

    def dxm1(self):
        ptr = self.L.orc_ctx_dxm1(self.hv)
        return np.ctypeslib.as_array(ptr, shape=(self.nx1 * self.nx1,)).copy()

    def wxm1(self):
        ptr = self.L.orc_ctx_wxm1(self.hv)
        return np.ctypeslib.as_array(ptr, shape=(self.nx1,)).copy()

    def set_threads(self, nthreads: int) -> None:
        self.L.orc_ctx_set_threads(self.hv, C.c_int(nthreads))

    def setup_g(self):
        g = np.zeros(6 * self.n)
        self.L.orc_setup_g(self.hv, _p(g))
        return g

    def set_multiplicity(self):
        c = np.zeros(self.n)
        self.L.orc_set_multiplicity(self.hv, _p(c))
        return c

    def set_f(self, c):
        f = np.zeros(self.n)
        self.L.orc_set_f(self.hv, _p(f), _p(c))
        return f

    def dssum(self, f):
        self.L.orc_dssum(self.hv, _p(f))

    def maskit(self, w):
        self.L.orc_maskit(self.hv, _p(w))

    def reset_mask(self):
        self.L.orc_ctx_reset_mask(self.hv)

    def ax(self, u, g):
        w = np.zeros(self.n)
        self.L.orc_ax(self.hv, _p(w), _p(np.ascontiguousarray(u)), _p(g))
        return w

    def ax_local(self, u, g):
        w = np.zeros(self.n)
        self.L.orc_ax_local(self.hv, _p(w), _p(np.ascontiguousarray(u)), _p(g))
        return w

    def cg(self, f, g, c, niter, use_mg=False, work=None):
        n = self.n
        x, r, w, p, z = work if work is not None else tuple(np.zeros(n) for _ in range(5))
        hist = np.zeros(5 * (niter + 1))
        it = self.L.orc_cg(self.hv, _p(x), _p(f), _p(g), _p(c), _p(r), _p(w), _p(p), _p(z),
                           C.c_int(n), C.c_int(niter), C.c_int(1 if use_mg else 0), _p(hist))
        return dict(x=x, r=r, w=w, p=p, z=z, hist=hist.reshape(niter + 1, 5), iter=it)

    def flops(self):
        return self.L.orc_flop_a(self.hv), self.L.orc_flop_cg(self.hv)

    def h1mg_setup(self, orders=None):
        if orders is None:
            return self.L.orc_h1mg_setup(self.hv, None, C.c_int(0))
        o = np.ascontiguousarray(orders, dtype=np.int32)
        return self.L.orc_h1mg_setup(self.hv, _p(o), C.c_int(len(o)))

    def h1mg_solve(self, rhs):
        z = np.zeros(self.n)
        self.L.orc_h1mg_solve(self.hv, _p(z), _p(rhs), C.c_int(self.n))
        return z

    def h1mg_levels(self):
        nl = self.L.orc_h1mg_nlev(self.hv)
        return [self.L.orc_h1mg_order(self.hv, C.c_int(l)) for l in range(1, nl + 1)]

    def fdm(self, l):
        order = self.h1mg_levels()[l - 1]
        nl = order + 3
        s = np.zeros(nl * nl * 6 * self.nelt)
        d = np.zeros(nl ** 3 * self.nelt)
        self.L.orc_h1mg_fdm_copy(self.hv, C.c_int(l), _p(s), _p(d))
        return s, d

    def __del__(self):
        try:
            self.L.orc_ctx_free(self.hv)
        except Exception:
            pass

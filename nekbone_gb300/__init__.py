"""nekbone_gb300 -- GB300 (sm_103a) implementation of Nekbone's spectral-element
Poisson CG hot path behind the reference's own routine interface.

The native library ``libnekbone_gb300.so`` (CUDA kernels + C ABI, see
``include/nekbone_gb300.h``) does all the work.  This module is the host-side
mirror of the reference's Fortran-callable routines -- same names, argument
meaning and error behaviour -- for callers that drive the hot path from
Python, and a thin wrapper of the device-resident ``nb_*`` API.

There is no fallback: importing the package loads the native library and
raises ``ImportError`` when it has not been built
(``python -m nekbone_gb300.build``).
"""
from __future__ import annotations

import ctypes as _C
from pathlib import Path as _Path

import numpy as _np

_LIB_PATH = _path = _Path(__file__).resolve().parent / "libnekbone_gb300.so"

if not _LIB_PATH.exists():
    raise ImportError(
        f"nekbone_gb300 native library missing at {_LIB_PATH}; build it with "
        "'python -m nekbone_gb300.build' (requires nvcc)")

lib = _C.CDLL(str(_LIB_PATH))

#: the library's default FP64 operator form (nekbone_set_contraction_order_)
DEFAULT_ORDER = 2

_i = _C.c_int
_l = _C.c_long
_d = _C.c_double
_p = _C.c_void_p
_ip = _C.POINTER(_C.c_int)
_dp = _C.POINTER(_C.c_double)

#: every symbol include/nekbone_gb300.h declares
EXPORTS = (
    "nekbone_last_status", "nekbone_last_message", "nekbone_clear_status",
    "nekbone_set_error_mode", "nekbone_version", "nekbone_common_",
    "nekbone_mask_reset_", "nekbone_set_mask_mode_", "nekbone_set_mgrid_",
    "nekbone_get_flops_", "nekbone_set_flops_", "nekbone_set_contraction_order_",
    "nb_mesh_set_order", "nb_setup_g_deformed", "nb_ax_f32", "nb_mg_setup",
    "nb_mg_solve", "nb_pcg_tol", "nb_tc_selftest", "nb_ax_tc", "gs_setup_", "gs_op_",
    "gs_free_", "dssum_", "glsc3_", "add2s1_", "add2s2_", "mxm_", "cg_", "ax_",
    "ax_e_", "local_grad3_", "local_grad3_t_", "maskit_", "solvem_",
    "h1mg_setup_", "h1mg_solve_", "zwgll_", "semhat_", "set_vert_box_",
    "cubic_", "get_exyz_", "setup_g_", "set_multiplicity_", "set_f_", "nb_mesh_create",
    "nb_mesh_destroy", "nb_mesh_npts", "nb_mesh_info", "nb_setup_g",
    "nb_set_multiplicity", "nb_rhs_uniform", "nb_ax", "nb_dssum", "nb_cg",
    "nb_cg_f32", "nb_cg_mixed", "nb_cg_tol", "nb_sync", "nb_stream",
    "nb_time_cg_kernels", "nb_glsc3_noalloc", "nb_time_cg_kernels_f32",
    "nb_batch_create", "nb_batch_destroy", "nb_batch_info", "nb_batch_problem",
    "nb_batch_arrays", "nb_batch_setup", "nb_batch_tune", "nb_batch_get_tuning",
    "nb_batch_set_tuning", "nb_batch_solve", "nb_batch_time_phases", "nb_batch_set_inner_tol", "nb_batch_result", "nb_batch_cycles",
    "nb_batch_rhs_in", "nb_batch_x_out", "nb_set_setup_on_device", "nb_set_mg_fixed_kernels", "nb_set_shared_metric", "nb_mesh_gs_maps",
    "nb_mesh_boundary_groups", "nb_mesh_mask_list", "nekbone_cg_report_",
    "nb_mg_setup_coarse", "nb_eo_line_maps", "nb_set_mixed_tensor_cores",
    "nb_set_paired_update", "nb_set_mixed_closed_multiplicity",
    "nb_wait_selftest", "nb_set_wait_test", "nb_pipe_rates",
)

lib.nekbone_last_status.restype = _i
lib.nekbone_last_message.restype = _C.c_char_p
lib.glsc3_.restype = _d
lib.nb_mesh_npts.restype = _l
for _name in ("nb_mesh_create", "nb_mesh_destroy", "nb_mesh_info", "nb_setup_g",
              "nb_set_multiplicity", "nb_rhs_uniform", "nb_ax", "nb_dssum", "nb_cg",
              "nb_cg_f32", "nb_cg_mixed", "nb_cg_tol", "nb_sync"):
    getattr(lib, _name).restype = _i
lib.nb_mesh_npts.argtypes = [_p]
lib.nb_tc_selftest.restype = _i
lib.nb_tc_selftest.argtypes = [_i, _p]
lib.nb_mg_setup.restype = _i
lib.nb_mg_setup.argtypes = [_p, _p, _i, _i]
lib.nb_mg_solve.restype = _i
lib.nb_mg_solve.argtypes = [_p, _p, _p]
lib.nb_pcg_tol.restype = _i
lib.nb_pcg_tol.argtypes = [_p, _p, _p, _p, _p, _d, _i, _i, _p, _p]
lib.nb_setup_g_deformed.restype = _i
lib.nb_setup_g_deformed.argtypes = [_p, _p, _C.c_uint64, _d]
lib.nb_ax_tc.restype = _i
lib.nb_ax_tc.argtypes = [_p, _p, _p, _p]
lib.nb_ax_f32.restype = _i
lib.nb_ax_f32.argtypes = [_p, _p, _p, _p]
lib.nb_mesh_set_order.restype = _i
lib.nb_mesh_set_order.argtypes = [_p, _i]
lib.nb_mesh_destroy.argtypes = [_p]
lib.nb_rhs_uniform.argtypes = [_p, _p, _p, _C.c_uint64]
lib.nb_cg.argtypes = [_p, _p, _p, _p, _p, _p, _p, _p, _p, _i, _i, _p]
lib.nb_cg_f32.argtypes = [_p, _p, _p, _p, _p, _p, _p, _p, _i, _p]
lib.nb_cg_mixed.argtypes = [_p, _p, _p, _p, _p, _d, _i, _i, _p, _p, _p]
lib.nb_cg_tol.argtypes = [_p, _p, _p, _p, _p, _d, _i, _i, _p, _p]
lib.nb_ax.argtypes = [_p, _p, _p, _p]
lib.nb_dssum.argtypes = [_p, _p, _i]
lib.nb_setup_g.argtypes = [_p, _p]
lib.nb_set_multiplicity.argtypes = [_p, _p]
lib.nb_mesh_info.argtypes = [_p, _p, _p, _p]
lib.nb_stream.restype = _p
lib.nb_time_cg_kernels.restype = _i
lib.nb_time_cg_kernels.argtypes = [_p, _p, _p, _p, _p, _p, _p, _p, _i, _p]
lib.nb_time_cg_kernels_f32.restype = _i
lib.nb_time_cg_kernels_f32.argtypes = [_p, _p, _p, _p, _p, _p, _p, _p, _i, _p]
lib.nb_glsc3_noalloc.restype = _i
lib.nb_glsc3_noalloc.argtypes = [_p, _p, _p, _l, _p, _p]
for _name, _args in (
        ("nb_batch_create", [_p, _i, _p, _p, _p, _p]),
        ("nb_batch_destroy", [_p]),
        ("nb_batch_info", [_p, _p, _p, _p]),
        ("nb_batch_problem", [_p, _i, _p, _p, _p]),
        ("nb_batch_arrays", [_p, _p, _p, _p, _p]),
        ("nb_batch_setup", [_p, _C.c_uint64]),
        ("nb_batch_tune", [_p, _i]),
        ("nb_batch_get_tuning", [_p, _i, _p, _p, _p, _p, _p]),
        ("nb_batch_set_tuning", [_p, _i, _i, _i, _i]),
        ("nb_batch_solve", [_p, _d, _i, _i]),
        ("nb_batch_time_phases", [_p, _d, _i, _i, _p, _p]),
        ("nb_batch_set_inner_tol", [_p, _d]),
        ("nb_batch_result", [_p, _i, _p, _p, _p]),
        ("nb_batch_cycles", [_p, _p]),
        ("nb_batch_rhs_in", [_p, _p]),
        ("nb_batch_x_out", [_p, _p])):
    getattr(lib, _name).restype = _i
    getattr(lib, _name).argtypes = _args
lib.nb_set_setup_on_device.restype = None
lib.nb_set_setup_on_device.argtypes = [_i]
lib.nb_set_mg_fixed_kernels.restype = None
lib.nb_set_mg_fixed_kernels.argtypes = [_i]
lib.nb_set_shared_metric.restype = None
lib.nb_set_shared_metric.argtypes = [_i]
lib.nb_set_mixed_tensor_cores.restype = None
lib.nb_set_mixed_tensor_cores.argtypes = [_i]
lib.nb_set_paired_update.restype = None
lib.nb_set_paired_update.argtypes = [_i]
lib.nb_set_mixed_closed_multiplicity.restype = None
lib.nb_set_mixed_closed_multiplicity.argtypes = [_i]
lib.nb_wait_selftest.restype = _i
lib.nb_wait_selftest.argtypes = [_C.c_uint]
lib.nb_set_wait_test.restype = _i
lib.nb_set_wait_test.argtypes = [_i]
lib.nb_pipe_rates.restype = _i
lib.nb_pipe_rates.argtypes = [_p]
for _name in ("nb_mesh_gs_maps", "nb_mesh_boundary_groups"):
    getattr(lib, _name).restype = _i
    getattr(lib, _name).argtypes = [_p, _p, _p, _p, _p]
lib.nb_mg_setup_coarse.restype = _i
lib.nb_mg_setup_coarse.argtypes = [_p, _p]
lib.nb_mesh_mask_list.restype = _i
lib.nb_mesh_mask_list.argtypes = [_p, _p, _p]
lib.nb_eo_line_maps.restype = _i
lib.nb_eo_line_maps.argtypes = [_i, _p, _p, _p]
#: largest n nb_glsc3_noalloc accepts (its fixed scratch holds the partials)
NOALLOC_MAX_N = 67108864

# return-status error mode for Python callers: errors raise NekboneError
lib.nekbone_set_error_mode(1)


class NekboneError(RuntimeError):
    """A failed library call; ``status`` is the library's status code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


def _check(ret: int | None = None) -> None:
    st = lib.nekbone_last_status() if ret is None else ret
    if st:
        msg = lib.nekbone_last_message().decode(errors="replace")
        lib.nekbone_clear_status()
        raise NekboneError(st, msg)


def _ref(v, t=_C.c_int):
    return _C.byref(t(v))


def _ptr(a: _np.ndarray):
    return a.ctypes.data_as(_p)


def _f64(a) -> _np.ndarray:
    a = _np.asarray(a)
    if a.dtype != _np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a


# ------------------------------------------------------------ set-up path --
def zwgll(np_: int):
    """GLL points and weights (speclib.f ZWGLL)."""
    z = _np.zeros(np_)
    w = _np.zeros(np_)
    lib.zwgll_(_ptr(z), _ptr(w), _ref(np_))
    return z, w


def semhat(n: int):
    """1-D matrices of degree n (semhat.f): a, b, c, d, z (d column-major)."""
    np_ = n + 1
    a, c, d = (_np.zeros(np_ * np_) for _ in range(3))
    b, z, w = _np.zeros(np_), _np.zeros(np_), _np.zeros(2 * np_)
    lib.semhat_(_ptr(a), _ptr(b), _ptr(c), _ptr(d), _ptr(z), _ptr(w), _ref(n))
    return a, b, c, d, z


def cubic(np_: int):
    """Most cube-like factorisation np = mx*my*mz (driver.f cubic)."""
    mx, my, mz = _C.c_int(), _C.c_int(), _C.c_int()
    lib.cubic_(_C.byref(mx), _C.byref(my), _C.byref(mz), _ref(np_))
    return mx.value, my.value, mz.value


def get_exyz(eg: int, nelx: int, nely: int, nelz: int):
    """Brick position (ex, ey, ez), 1-based, of global element eg
    (prox_dssum.f get_exyz)."""
    ex, ey, ez = _C.c_int(), _C.c_int(), _C.c_int()
    lib.get_exyz_(_C.byref(ex), _C.byref(ey), _C.byref(ez), _ref(eg), _ref(nelx),
                  _ref(nely), _ref(nelz))
    return ex.value, ey.value, ez.value


# ----------------------------------------------------------- gather-scatter --
_DOM = {_np.dtype(_np.float64): 1, _np.dtype(_np.float32): 2,
        _np.dtype(_np.int32): 3, _np.dtype(_np.int64): 4}


def gs_setup(glo_num) -> int:
    """gs_setup (jl/gs.c:1160): handle for the global numbering glo_num."""
    ids = _np.ascontiguousarray(glo_num, dtype=_np.int64)
    h = _C.c_int(-1)
    lib.gs_setup_(_C.byref(h), _ptr(ids), _ref(len(ids)), _ref(0), _ref(1))
    _check()
    return h.value


def gs_op(handle: int, u: _np.ndarray, op: int = 1, transpose: int = 0) -> None:
    """gs_op (jl/gs.c:1188) in place; the dom follows u's dtype."""
    dom = _DOM.get(u.dtype)
    if dom is None or not u.flags.c_contiguous:
        raise TypeError("u must be a C-contiguous float64/float32/int32/int64 array")
    lib.gs_op_(_ref(handle), _ptr(u), _ref(dom), _ref(op), _ref(transpose))
    _check()


def gs_free(handle: int) -> None:
    lib.gs_free_(_ref(handle))
    _check()


# --------------------------------------------------------------- math.f --
def glsc3(a, b, mult) -> float:
    a, b, mult = _f64(a), _f64(b), _f64(mult)
    v = lib.glsc3_(_ptr(a), _ptr(b), _ptr(mult), _ref(len(a)))
    _check()
    return v


def add2s1(a, b, c1: float) -> None:
    a, b = _f64(a), _f64(b)
    lib.add2s1_(_ptr(a), _ptr(b), _ref(c1, _C.c_double), _ref(len(a)))
    _check()


def add2s2(a, b, c1: float) -> None:
    a, b = _f64(a), _f64(b)
    lib.add2s2_(_ptr(a), _ptr(b), _ref(c1, _C.c_double), _ref(len(a)))
    _check()


def mxm(a, n1: int, b, n2: int, n3: int) -> _np.ndarray:
    a, b = _f64(a), _f64(b)
    c = _np.zeros(n1 * n3)
    lib.mxm_(_ptr(a), _ref(n1), _ptr(b), _ref(n2), _ptr(c), _ref(n3))
    _check()
    return c


def local_grad3(u, n: int, D, Dt):
    m3 = (n + 1) ** 3
    ur, us, ut = _np.zeros(m3), _np.zeros(m3), _np.zeros(m3)
    lib.local_grad3_(_ptr(ur), _ptr(us), _ptr(ut), _ptr(_f64(u)), _ref(n),
                     _ptr(_f64(D)), _ptr(_f64(Dt)))
    _check()
    return ur, us, ut


def local_grad3_t(ur, us, ut, n: int, D, Dt):
    m3 = (n + 1) ** 3
    u, w = _np.zeros(m3), _np.zeros(m3)
    lib.local_grad3_t_(_ptr(u), _ptr(_f64(ur)), _ptr(_f64(us)), _ptr(_f64(ut)),
                       _ref(n), _ptr(_f64(D)), _ptr(_f64(Dt)), _ptr(w))
    _check()
    return u, w


# ------------------------------------------------------------ driver level --
class Nekbone:
    """The Fortran driver's view of one mesh (driver.f:38-67): publishes the
    common blocks and calls the drop-in routines with host arrays.

    mask_mode 0 reproduces the reference's maskit (after the first call only
    element 1's Dirichlet points are zeroed, cg.f:224-229); 1 masks every
    element's outer faces.
    """

    def __init__(self, nelx: int, nely: int, nelz: int, nx1: int,
                 mask_mode: int = 0, lglel=None):
        self.nelx, self.nely, self.nelz, self.nx1 = nelx, nely, nelz, nx1
        self.nelt = nelx * nely * nelz
        self.n = self.nelt * nx1 ** 3
        self.lglel = (_np.arange(1, self.nelt + 1, dtype=_np.int32) if lglel is None
                      else _np.ascontiguousarray(lglel, dtype=_np.int32))
        _, _, _, d, z = semhat(nx1 - 1)
        self.dxm1 = d
        lib.nekbone_set_mask_mode_(_ref(mask_mode))
        _check()
        # publish /dimn/ and /hcglb/ so set_vert_box can run, then gs_setup
        lib.nekbone_common_(_ref(nelx), _ref(nely), _ref(nelz), _ref(self.nelt),
                            _ref(nx1), _ptr(self.lglel), _ptr(self.dxm1), _ref(-1))
        _check()
        self.glo_num = _np.zeros(self.n, dtype=_np.int64)
        lib.set_vert_box_(_ptr(self.glo_num), _ref(nx1))
        _check()
        self.gsh = gs_setup(self.glo_num)
        lib.nekbone_common_(_ref(nelx), _ref(nely), _ref(nelz), _ref(self.nelt),
                            _ref(nx1), _ptr(self.lglel), _ptr(self.dxm1), _ref(self.gsh))
        _check()

    def set_multiplicity(self) -> _np.ndarray:
        c = _np.zeros(self.n)
        lib.set_multiplicity_(_ptr(c))
        _check()
        return c

    def setup_g(self) -> _np.ndarray:
        g = _np.zeros(6 * self.n)
        lib.setup_g_(_ptr(g))
        _check()
        return g

    def set_f(self, c) -> _np.ndarray:
        f = _np.zeros(self.n)
        lib.set_f_(_ptr(f), _ptr(_f64(c)), _ref(self.n))
        _check()
        return f

    def dssum(self, f) -> None:
        lib.dssum_(_ptr(_f64(f)))
        _check()

    def mask_reset(self) -> None:
        lib.nekbone_mask_reset_()

    @staticmethod
    def set_order(order: int) -> None:
        """0 = reference left-to-right contraction sums, 1 = even-odd split
        on the FP64 pipe, 2 = even-odd in 64-bit fixed point (DEFAULT_ORDER)."""
        lib.nekbone_set_contraction_order_(_ref(order))
        _check()

    def set_mgrid(self, on: bool) -> None:
        lib.nekbone_set_mgrid_(_ref(1 if on else 0))

    def h1mg_setup(self) -> None:
        lib.h1mg_setup_()
        _check()

    def h1mg_solve(self, rhs) -> _np.ndarray:
        z = _np.zeros(self.n)
        lib.h1mg_solve_(_ptr(z), _ptr(_f64(rhs)), _ref(self.n))
        _check()
        return z

    def ax(self, u, g) -> _np.ndarray:
        w = _np.zeros(self.n)
        s = _np.zeros(1)
        lib.ax_(_ptr(w), _ptr(_f64(u)), _ptr(_f64(g)), _ptr(s), _ptr(s), _ptr(s), _ptr(s),
                _ref(self.n))
        _check()
        return w

    def ax_e(self, u, g) -> _np.ndarray:
        m3 = self.nx1 ** 3
        w, s = _np.zeros(m3), _np.zeros(1)
        lib.ax_e_(_ptr(w), _ptr(_f64(u)), _ptr(_f64(g)), _ptr(s), _ptr(s), _ptr(s), _ptr(s))
        _check()
        return w

    def maskit(self, w, pmask) -> None:
        lib.maskit_(_ptr(_f64(w)), _ptr(_f64(pmask)), _ref(self.nx1), _ref(self.nx1),
                    _ref(self.nx1))
        _check()

    def cg(self, f, g, c, niter: int, flop_cg: float = 0.0, work=None):
        """cg (cg.f:2-84).  Returns x, r, w, p, z, flop_cg."""
        n = self.n
        x, r, w, p, z = work if work is not None else tuple(_np.zeros(n) for _ in range(5))
        fc = _C.c_double(flop_cg)
        lib.cg_(_ptr(x), _ptr(_f64(f)), _ptr(_f64(g)), _ptr(_f64(c)), _ptr(r), _ptr(w),
                _ptr(p), _ptr(z), _ref(n), _ref(niter), _C.byref(fc))
        _check()
        return x, r, w, p, z, fc.value

    @staticmethod
    def flops():
        a, c = _C.c_double(), _C.c_double()
        lib.nekbone_get_flops_(_C.byref(a), _C.byref(c))
        return a.value, c.value

    @staticmethod
    def set_flops(a: float, c: float) -> None:
        lib.nekbone_set_flops_(_ref(a, _C.c_double), _ref(c, _C.c_double))


# ------------------------------------------------------------ device API --
class DeviceMesh:
    """Box mesh resident on the GPU (the nb_* API).  Vectors are passed as
    raw device pointers (ints), e.g. ``torch.Tensor.data_ptr()``."""

    def __init__(self, nelx: int, nely: int, nelz: int, lx1: int, mask_mode: int = 1):
        h = _p()
        _check(lib.nb_mesh_create(_C.byref(h), nelx, nely, nelz, lx1, mask_mode))
        self._h = h
        self.n = int(lib.nb_mesh_npts(h))
        nelt, lx, fused = _C.c_int(), _C.c_int(), _C.c_int()
        _check(lib.nb_mesh_info(h, _C.byref(nelt), _C.byref(lx), _C.byref(fused)))
        self.nelt, self.lx1, self.fused = nelt.value, lx.value, bool(fused.value)
        self.dims = (nelx, nely, nelz)

    def close(self) -> None:
        if self._h:
            lib.nb_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def gs_maps(self):
        """(off, idx) of the gather-scatter groups (int32 numpy arrays)."""
        ng, nm = _C.c_int(), _C.c_long()
        _check(lib.nb_mesh_gs_maps(self._h, _C.byref(ng), _C.byref(nm), None, None))
        off = _np.zeros(ng.value + 1, dtype=_np.int32)
        idx = _np.zeros(max(nm.value, 1), dtype=_np.int32)
        _check(lib.nb_mesh_gs_maps(self._h, None, None, _ptr(off), _ptr(idx)))
        return off, idx[:nm.value]

    def boundary_groups(self):
        """(off, idx) of the fused boundary groups (idx uint32, bit 31 = masked)."""
        ng, nm = _C.c_int(), _C.c_long()
        _check(lib.nb_mesh_boundary_groups(self._h, _C.byref(ng), _C.byref(nm), None, None))
        off = _np.zeros(ng.value + 1, dtype=_np.int32)
        idx = _np.zeros(max(nm.value, 1), dtype=_np.uint32)
        _check(lib.nb_mesh_boundary_groups(self._h, None, None, _ptr(off), _ptr(idx)))
        return off, idx[:nm.value]

    def mask_list(self):
        n = _C.c_int()
        _check(lib.nb_mesh_mask_list(self._h, _C.byref(n), None))
        out = _np.zeros(max(n.value, 1), dtype=_np.int32)
        _check(lib.nb_mesh_mask_list(self._h, None, _ptr(out)))
        return out[:n.value]

    def set_order(self, order: int) -> None:
        _check(lib.nb_mesh_set_order(self._h, order))

    def setup_g(self, g_ptr: int) -> None:
        _check(lib.nb_setup_g(self._h, _p(g_ptr)))

    def setup_g_deformed(self, g_ptr: int, seed: int, amp: float = 0.1) -> None:
        _check(lib.nb_setup_g_deformed(self._h, _p(g_ptr), seed, amp))

    def ax_tc(self, w_ptr: int, u_ptr: int, g_ptr: int) -> None:
        _check(lib.nb_ax_tc(self._h, _p(w_ptr), _p(u_ptr), _p(g_ptr)))

    def ax_f32(self, w_ptr: int, u_ptr: int, g_ptr: int) -> None:
        _check(lib.nb_ax_f32(self._h, _p(w_ptr), _p(u_ptr), _p(g_ptr)))

    def set_multiplicity(self, c_ptr: int) -> None:
        _check(lib.nb_set_multiplicity(self._h, _p(c_ptr)))

    def rhs_uniform(self, f_ptr: int, c_ptr: int, seed: int) -> None:
        _check(lib.nb_rhs_uniform(self._h, _p(f_ptr), _p(c_ptr), seed))

    def ax(self, w_ptr: int, u_ptr: int, g_ptr: int) -> None:
        _check(lib.nb_ax(self._h, _p(w_ptr), _p(u_ptr), _p(g_ptr)))

    def dssum(self, u_ptr: int, dom: int = 1) -> None:
        _check(lib.nb_dssum(self._h, _p(u_ptr), dom))

    def cg(self, x, f, g, c, r, w, p, z, niter: int, flags: int = 0, hist: bool = False):
        h = _np.zeros(5 * (niter + 1)) if hist else None
        _check(lib.nb_cg(self._h, _p(x), _p(f), _p(g), _p(c), _p(r), _p(w), _p(p), _p(z),
                         niter, flags, _ptr(h) if hist else None))
        return h.reshape(niter + 1, 5) if hist else None

    def cg_f32(self, x, f, g, c, r, w, p, niter: int, hist: bool = False):
        h = _np.zeros(5 * (niter + 1)) if hist else None
        _check(lib.nb_cg_f32(self._h, _p(x), _p(f), _p(g), _p(c), _p(r), _p(w), _p(p),
                             niter, _ptr(h) if hist else None))
        return h.reshape(niter + 1, 5) if hist else None

    def cg_mixed(self, x, f, g, c, tol: float, inner_iters: int = 20, max_outer: int = 500):
        o, it, rr = _C.c_int(), _C.c_int(), _C.c_double()
        _check(lib.nb_cg_mixed(self._h, _p(x), _p(f), _p(g), _p(c), tol, inner_iters,
                               max_outer, _C.byref(o), _C.byref(it), _C.byref(rr)))
        return o.value, it.value, rr.value

    def time_cg_kernels(self, x, f, g, c, r, w, p, reps: int = 10):
        ms = _np.zeros(3)
        _check(lib.nb_time_cg_kernels(self._h, _p(x), _p(f), _p(g), _p(c), _p(r), _p(w),
                                      _p(p), reps, _ptr(ms)))
        return ms

    def time_cg_kernels_f32(self, x, f, g, c, r, w, p, reps: int = 10):
        ms = _np.zeros(3)
        _check(lib.nb_time_cg_kernels_f32(self._h, _p(x), _p(f), _p(g), _p(c), _p(r),
                                          _p(w), _p(p), reps, _ptr(ms)))
        return ms

    def mg_setup(self, orders=None, precision: int = 64) -> None:
        if orders is None:
            _check(lib.nb_mg_setup(self._h, None, 0, precision))
        else:
            o = _np.ascontiguousarray(orders, dtype=_np.int32)
            _check(lib.nb_mg_setup(self._h, _ptr(o), len(o), precision))

    def mg_setup_coarse(self, g) -> None:
        """Exact Galerkin coarse solve for metric g (after mg_setup)."""
        _check(lib.nb_mg_setup_coarse(self._h, _p(g)))

    def mg_solve(self, z, rhs) -> None:
        _check(lib.nb_mg_solve(self._h, _p(z), _p(rhs)))

    def pcg_tol(self, x, f, g, c, tol: float, max_iter: int = 5000, check_every: int = 5):
        it, rr = _C.c_int(), _C.c_double()
        _check(lib.nb_pcg_tol(self._h, _p(x), _p(f), _p(g), _p(c), tol, max_iter,
                              check_every, _C.byref(it), _C.byref(rr)))
        return it.value, rr.value

    def cg_tol(self, x, f, g, c, tol: float, max_iter: int = 20000, check_every: int = 25):
        it, rr = _C.c_int(), _C.c_double()
        _check(lib.nb_cg_tol(self._h, _p(x), _p(f), _p(g), _p(c), tol, max_iter,
                             check_every, _C.byref(it), _C.byref(rr)))
        return it.value, rr.value


class Batch:
    """Many independent box-mesh problems solved together (nb_batch_*).

    ``boxes`` is a sequence of (nelx, nely, nelz, lx1).  Device vectors of
    problem p live at ``offset(p)`` in the concatenated arrays whose device
    pointers ``arrays()`` returns."""

    def __init__(self, boxes):
        boxes = [tuple(int(v) for v in b) for b in boxes]
        self.nprob = len(boxes)
        col = [_np.ascontiguousarray([b[k] for b in boxes], dtype=_np.int32) for k in range(4)]
        h = _C.c_void_p()
        _check(lib.nb_batch_create(_C.byref(h), self.nprob, *[_ptr(c) for c in col]))
        self._h = h
        self.boxes = boxes
        n, ne, nl = _C.c_long(), _C.c_int(), _C.c_int()
        _check(lib.nb_batch_info(self._h, _C.byref(n), _C.byref(ne), _C.byref(nl)))
        self.n, self.nelt, self.nlx = n.value, ne.value, nl.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.nb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def problem(self, p: int):
        """(point offset, number of points, lx1) of problem p"""
        o, n, l = _C.c_long(), _C.c_long(), _C.c_int()
        _check(lib.nb_batch_problem(self._h, p, _C.byref(o), _C.byref(n), _C.byref(l)))
        return o.value, n.value, l.value

    def arrays(self):
        """device pointers (x, f, g, c)"""
        ptrs = [_C.c_void_p() for _ in range(4)]
        _check(lib.nb_batch_arrays(self._h, *[_C.byref(q) for q in ptrs]))
        return tuple(q.value for q in ptrs)

    def setup(self, seed: int) -> None:
        _check(lib.nb_batch_setup(self._h, _C.c_uint64(seed)))

    def tune(self, reps: int = 3) -> None:
        _check(lib.nb_batch_tune(self._h, reps))

    def tuning(self, lx: int):
        e32, r32, e64 = _C.c_int(), _C.c_int(), _C.c_int()
        m32, m64 = _C.c_float(), _C.c_float()
        _check(lib.nb_batch_get_tuning(self._h, lx, _C.byref(e32), _C.byref(r32), _C.byref(e64),
                                       _C.byref(m32), _C.byref(m64)))
        return {"epb32": e32.value, "rd32": r32.value, "epb64": e64.value,
                "ms32": m32.value, "ms64": m64.value}

    def set_tuning(self, lx: int, epb32: int, rd32: int, epb64: int) -> None:
        _check(lib.nb_batch_set_tuning(self._h, lx, epb32, rd32, epb64))

    def set_inner_tol(self, itol: float) -> None:
        """0: fixed inner_iters per cycle; > 0: each problem's inner CG stops
        once its residual fell by itol (at most inner_iters)"""
        _check(lib.nb_batch_set_inner_tol(self._h, _C.c_double(itol)))

    def solve(self, tol: float = 1e-10, inner_iters: int = 20, max_outer: int = 50) -> None:
        """enqueue the whole solve (one graph launch) on the library stream"""
        _check(lib.nb_batch_solve(self._h, _C.c_double(tol), inner_iters, max_outer))

    PHASES = ("init", "scale", "inner_ax", "inner_gs_dot", "inner_update", "defect_ax",
              "defect_gs_residual")

    def time_phases(self, tol: float = 1e-10, inner_iters: int = 20, max_outer: int = 50):
        """The solve launched one cycle at a time with an event after every
        kernel (same kernels, same results; synchronous): ({phase: ms summed
        over the solve}, cycles)"""
        ms = (_C.c_double * len(self.PHASES))()
        cyc = _C.c_int()
        _check(lib.nb_batch_time_phases(self._h, _C.c_double(tol), inner_iters, max_outer, ms,
                                        _C.byref(cyc)))
        return dict(zip(self.PHASES, list(ms))), cyc.value

    def result(self, p: int):
        """(cycles, inner iterations, |r|_C/|f|_C) of problem p"""
        o, i, rr = _C.c_int(), _C.c_int(), _C.c_double()
        _check(lib.nb_batch_result(self._h, p, _C.byref(o), _C.byref(i), _C.byref(rr)))
        return o.value, i.value, rr.value

    def cycles(self) -> int:
        v = _C.c_int()
        _check(lib.nb_batch_cycles(self._h, _C.byref(v)))
        return v.value

    def rhs_in(self, host_ptr: int) -> None:
        _check(lib.nb_batch_rhs_in(self._h, _C.c_void_p(host_ptr)))

    def x_out(self, host_ptr: int) -> None:
        _check(lib.nb_batch_x_out(self._h, _C.c_void_p(host_ptr)))


def set_setup_on_device(on: bool) -> None:
    """Build full-mask mesh topologies on the device (default) or the host."""
    lib.nb_set_setup_on_device(1 if on else 0)


def set_mg_fixed_kernels(on: bool) -> None:
    """hsmg: fixed-size FDM/transfer kernels (default) or the general ones."""
    lib.nb_set_mg_fixed_kernels(1 if on else 0)


def eo_line_maps(lx1: int):
    """The FP32 even-odd operator's line order for lx1: (plane stride,
    r-line map, s-line map); thread t takes r-line rmap[t] = j + lx1 k and
    s-line smap[t] = i + lx1 k."""
    pl = _C.c_int()
    r = _np.zeros(lx1 * lx1, dtype=_np.uint8)
    s_ = _np.zeros(lx1 * lx1, dtype=_np.uint8)
    _check(lib.nb_eo_line_maps(lx1, _C.byref(pl), _ptr(r), _ptr(s_)))
    return pl.value, r, s_


def set_mixed_tensor_cores(on: bool) -> None:
    """Mixed solver: the inner CG's element products on the tensor cores
    (True) or the fused CUDA-core iteration (False, default)."""
    lib.nb_set_mixed_tensor_cores(1 if on else 0)


def set_paired_update(on: bool) -> None:
    """FP64 CG (fused, no preconditioner), the mixed solver's inner FP32 CG
    and the batched solve's inner CG: x updated once per two iterations from
    two direction buffers (True, default) or every iteration (False);
    bitwise the same iterates."""
    lib.nb_set_paired_update(1 if on else 0)


def set_mixed_closed_multiplicity(on: bool) -> None:
    """Mixed solver: the inner FP32 CG forms c in closed form when c
    verifies as a box mesh's inverse multiplicity (True, default), or
    always reads it (False); bitwise the same iterates."""
    lib.nb_set_mixed_closed_multiplicity(1 if on else 0)


def set_shared_metric(on: bool) -> None:
    """Mixed solver: one shared FP32 metric block when all elements' are
    equal (default), or always each element's."""
    lib.nb_set_shared_metric(1 if on else 0)


def tc_selftest(bf16: bool = False) -> int:
    """Runs one tcgen05 MMA on known operands; returns the mismatch count."""
    bad = _C.c_int(-1)
    _check(lib.nb_tc_selftest(1 if bf16 else 0, _C.byref(bad)))
    return bad.value


def wait_selftest(polls: int = 256) -> None:
    """Runs a bounded wait that nothing completes; raises NekboneError with
    the status a timed-out device wait produces."""
    _check(lib.nb_wait_selftest(polls))


def set_wait_test(on: bool) -> None:
    """Makes the bulk-copy waits of later launches run out on purpose (the
    timeout path of the real kernels); off restores normal runs."""
    _check(lib.nb_set_wait_test(1 if on else 0))


def pipe_rates() -> dict:
    """Measured operations per second of the FP64 FMA, integer
    multiply-add (mad.wide.s32), integer add and FP32 FMA pipes."""
    r = _np.zeros(4)
    _check(lib.nb_pipe_rates(_ptr(r)))
    return {"dfma": float(r[0]), "imad_wide": float(r[1]), "iadd": float(r[2]),
            "ffma": float(r[3])}


def stream_handle() -> int:
    """cudaStream_t of the library (wrap with torch.cuda.ExternalStream)."""
    return int(lib.nb_stream() or 0)


def sync() -> None:
    _check(lib.nb_sync())

"""The reference's driver program against the library, call by call.

tests/golden/driver_trace_*.npz hold every call that driver.f's own `program
nekbone` (driver.f:2-86, run by the Fortran 77 executor over the reference's
sources; see make_golden_driver.py) makes into the routines the library
replaces, with the arguments as the program passed them and as the
reference's implementation returned them, plus the hand-off lines the link
step adds (nekbone_mask_reset after init_mesh; nekbone_common,
nekbone_set_mask_mode, nekbone_set_mgrid after proxy_setup).

Here the same calls, in the same order and with the same arguments, go to
the library's gfortran-convention symbols (gs_setup_, gs_op_, dssum_,
h1mg_setup_, cg_, gs_free_, ...) through ctypes, by reference, as a gfortran
link would make them.  The cases cover two polynomial orders (one below the
SIZE file's lx1) and two element counts, each mesh set up, solved twice and
freed, and the MGRID build.  Handles are the library's own, mapped from the
recorded ones.

Tolerances: gather-scatter results (set_multiplicity's gs_op, set_f's dssum)
are bit-exact; cg's x and r after 100 iterations agree to 1e-12 (relative to
max|x| and max|f|: the library sums dot products in a tree, the reference
sequentially); flop_cg is exact.  Every FP64 operator form runs.
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden"
TRACES = sorted(GOLDEN.glob("driver_trace_*.npz"))


@pytest.fixture(scope="module")
def lib():
    import nekbone_gb300 as nb
    # a second handle on the loaded library: prototypes set here stay here
    L = C.CDLL(str(nb._LIB_PATH))
    L.nekbone_last_status.restype = C.c_int
    L.nekbone_last_message.restype = C.c_char_p
    L.nekbone_set_error_mode(1)
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _check(L, what):
    st = L.nekbone_last_status()
    assert st == 0, f"{what}: {L.nekbone_last_message().decode()}"


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("path", TRACES, ids=[p.stem for p in TRACES])
def test_driver_program_calls_match_reference(lib, path, order):
    L = lib
    z = np.load(path)
    calls = json.loads(str(z["calls"]))
    o = C.c_int(order)
    L.nekbone_set_contraction_order_(C.byref(o))
    handles = {}
    names = []
    try:
        for k, call in enumerate(calls):
            name = call["name"]
            names.append(name)
            a_in = [np.array(z[f"c{k}_a{j}_in"]) for j in range(len(call["kinds"]))]
            a_out = [z[f"c{k}_a{j}_out"] for j in range(len(call["kinds"]))]
            L.nekbone_clear_status()
            if name == "nekbone_mask_reset":
                L.nekbone_mask_reset_()
            elif name in ("nekbone_set_mask_mode", "nekbone_set_mgrid"):
                getattr(L, name + "_")(_ptr(a_in[0]))
            elif name == "nekbone_common":
                a_in[7] = np.array([handles[int(a_in[7][0])]], dtype=np.int32)
                L.nekbone_common_(*[_ptr(a) for a in a_in])
            elif name == "gs_setup":
                L.gs_setup_(*[_ptr(a) for a in a_in])
                handles[int(a_out[0][0])] = int(a_in[0][0])
            elif name == "gs_op":
                a_in[0][0] = handles[int(a_in[0][0])]
                L.gs_op_(*[_ptr(a) for a in a_in])
                _check(L, f"call {k} gs_op")
                assert np.array_equal(a_in[1], a_out[1]), f"call {k} gs_op"
            elif name == "dssum":
                L.dssum_(_ptr(a_in[0]))
                _check(L, f"call {k} dssum")
                assert np.array_equal(a_in[0], a_out[0]), f"call {k} dssum"
            elif name == "h1mg_setup":
                L.h1mg_setup_()
            elif name == "cg":
                L.cg_(*[_ptr(a) for a in a_in])
                _check(L, f"call {k} cg")
                x, r, f, flop = a_in[0], a_in[4], a_in[1], a_in[10]
                assert _rel(x, a_out[0]) < 1e-12, (k, _rel(x, a_out[0]))
                assert np.max(np.abs(r - a_out[4])) < 1e-12 * np.max(np.abs(f)), k
                assert flop[0] == a_out[10][0], (k, flop[0], a_out[10][0])
            elif name == "gs_free":
                a_in[0][0] = handles.pop(int(a_in[0][0]))
                L.gs_free_(_ptr(a_in[0]))
            else:
                raise AssertionError(f"unknown call {name}")
            _check(L, f"call {k} {name}")
    finally:
        import nekbone_gb300 as nb
        d = C.c_int(nb.DEFAULT_ORDER)
        L.nekbone_set_contraction_order_(C.byref(d))
        L.nekbone_set_mgrid_(C.byref(C.c_int(0)))
    assert names.count("cg") >= 2 and not handles

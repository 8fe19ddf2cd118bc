"""CPU tests of the native library: it loads, exports every symbol
include/nekbone_gb300.h declares, and its host-side set-up routines (which
run without a GPU) agree with the oracle bit for bit."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    src = (ROOT / "include" / "nekbone_gb300.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src)
    skip = {"if", "for", "while", "return", "sizeof", "defined"}
    return sorted({n for n in names if n not in skip})


def test_library_exports_header():
    import nekbone_gb300 as nb
    syms = header_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(nb.lib, s)]
    assert not missing, missing
    assert set(syms) == set(nb.EXPORTS)


@pytest.mark.parametrize("np_", [2, 3, 4, 5, 6, 8, 10, 12, 13, 16, 20])
def test_zwgll_matches_oracle(np_):
    import nekbone_gb300 as nb
    z, w = nb.zwgll(np_)
    zo, wo = O.zwgll(np_)
    assert np.array_equal(z, zo) and np.array_equal(w, wo)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 9, 11, 15])
def test_semhat_matches_oracle(n):
    import nekbone_gb300 as nb
    mine = nb.semhat(n)
    ref = O.semhat(n)
    for a, b in zip(mine, ref):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("np_", [1, 2, 7, 12, 50, 64, 100, 4096, 32768, 360])
def test_cubic_matches_oracle(np_):
    import nekbone_gb300 as nb
    assert nb.cubic(np_) == O.cubic(np_)


def test_error_mode_returns_status():
    import nekbone_gb300 as nb
    with pytest.raises(nb.NekboneError) as e:
        nb.gs_op(12345, np.zeros(3))
    assert e.value.status == 2          # NB_ERR_HANDLE
    with pytest.raises(nb.NekboneError):
        nb.lib.gs_op_(nb._ref(0), nb._ptr(np.zeros(1)), nb._ref(7), nb._ref(1), nb._ref(0))
        nb._check()


def test_reference_error_mode_exits_with_status_1(tmp_path):
    """Error mode 0 mirrors jl's fail(): print and exit(1) (jl/fail.c:11-52)."""
    import subprocess
    import sys
    code = ("import nekbone_gb300 as nb, numpy as np\n"
            "nb.lib.nekbone_set_error_mode(0)\n"
            "nb.lib.gs_free_(nb._ref(99))\n"
            "print('not reached')\n")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       cwd=str(ROOT))
    assert p.returncode == 1
    assert "invalid handle" in p.stderr
    assert "not reached" not in p.stdout


def test_batch_rejects_bad_problems_without_a_gpu():
    """nb_batch_create validates every problem before it touches the device."""
    import nekbone_gb300 as nb
    with pytest.raises(nb.NekboneError) as e:
        nb.Batch([(2, 2, 2, 6), (2, 2, 2, 5)])      # lx1=5 has no batched kernel
    assert e.value.status != 0
    with pytest.raises(nb.NekboneError):
        nb.Batch([(0, 2, 2, 6)])
    with pytest.raises(nb.NekboneError):
        nb.Batch([])


@pytest.mark.parametrize("dims", [(4, 4, 4), (3, 2, 5), (1, 1, 7), (6, 1, 1)])
def test_get_exyz_brick_positions(dims):
    """get_exyz (prox_dssum.f:75-86): element eg of the brick order sits at
    (ex, ey, ez) with eg = ex + nelx*(ey-1) + nelx*nely*(ez-1); every
    position once."""
    import nekbone_gb300 as nb
    nelx, nely, nelz = dims
    seen = set()
    for eg in range(1, nelx * nely * nelz + 1):
        ex, ey, ez = nb.get_exyz(eg, nelx, nely, nelz)
        assert 1 <= ex <= nelx and 1 <= ey <= nely and 1 <= ez <= nelz
        assert ex + nelx * (ey - 1) + nelx * nely * (ez - 1) == eg
        seen.add((ex, ey, ez))
    assert len(seen) == nelx * nely * nelz

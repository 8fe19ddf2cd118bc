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


def _warp_wavefronts(starts, nt):
    """Shared-memory wavefronts of one line phase: per warp, the most lines
    whose first words share a bank (4-byte words, 32 banks)."""
    total = 0
    for w in range(0, nt, 32):
        banks = {}
        for s in starts[w:w + 32]:
            banks[s % 32] = banks.get(s % 32, 0) + 1
        total += max(banks.values())
    return total


# (lx1, r-line wavefronts, s-line wavefronts) the dealt order reaches; the
# bound is one per warp where every bank holds at most one line per warp
DEALT_COST = [(2, 1, 1), (4, 1, 1), (6, 2, 3), (8, 2, 3), (10, 5, 5), (12, 5, 6)]


@pytest.mark.parametrize("lx,cr,cs", DEALT_COST)
def test_eo_line_maps_deal_lines_to_distinct_banks(lx, cr, cs):
    import nekbone_gb300 as nb
    pl, rmap, smap = nb.eo_line_maps(lx)
    nt = lx * lx
    assert pl >= lx * lx
    assert sorted(rmap.tolist()) == list(range(nt))
    assert sorted(smap.tolist()) == list(range(nt))
    # first word of r-line (j, k): j lx + k pl; of s-line (i, k): i + k pl
    rs = [(l % lx) * lx + (l // lx) * pl for l in rmap.tolist()]
    ss = [(l % lx) + (l // lx) * pl for l in smap.tolist()]
    assert _warp_wavefronts(rs, nt) <= cr
    assert _warp_wavefronts(ss, nt) <= cs
    # against the rows-padded layout in natural order, weighting each phase
    # by its accesses per point (7 column accesses, 4 r-line, 4 s-line)
    nat = list(range(nt))
    col_new = _warp_wavefronts(nat, nt)                 # thread (i, j): word i + lx j
    col_pad = _warp_wavefronts([(t % lx) + (t // lx) * (lx + 1) for t in nat], nt)
    r_pad = _warp_wavefronts([(l % lx) * (lx + 1) + (l // lx) * (lx + 1) * lx for l in nat], nt)
    s_pad = _warp_wavefronts([(l % lx) + (l // lx) * (lx + 1) * lx for l in nat], nt)
    assert col_new == (nt + 31) // 32
    assert 7 * col_new + 4 * (cr + cs) <= 7 * col_pad + 4 * (r_pad + s_pad)


def test_eo_line_maps_rejects_bad_orders():
    import nekbone_gb300 as nb
    for lx in (3, 14, 0):
        with pytest.raises(nb.NekboneError):
            nb.eo_line_maps(lx)

"""The oracle against the reference's own Fortran, run on small cases.

The fixtures tests/golden/fortran_*.npz come from the reference's Fortran
sources executed by oracle/f77.py (gfortran -fdefault-real-8 semantics, no
FMA contraction), with the reference's jl library for gather-scatter; see
tests/golden/make_golden_fortran.py.  They pin the oracle's restatement of:
GLL points (speclib.f), semhat (semhat.f), cubic (driver.f), set_vert_box
(prox_dssum.f), setup_g (prox_setup.f), set_multiplicity and set_f
(driver.f), ax with the reference's maskit (cg.f), cg -- the warm-up call and
the timed call with its element-1 mask list -- and hsmg.

Tolerances: the oracle's plain build (separate multiply and add) must equal
the reference bit for bit everywhere except hsmg.  hsmg's generalised
eigenproblems are solved by different eigensolvers (the oracle's Jacobi
method, LAPACK's dsygv for the reference), so its results agree to 1e-12
relative.  The oracle's FMA build (the order the GPU kernels follow) agrees
with the reference to rounding: 1e-13 relative after the CG iterations.
"""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O

GOLDEN = Path(__file__).parent / "golden"
BOXES = sorted(GOLDEN.glob("fortran_box_*.npz"))


def _load(name):
    p = GOLDEN / name
    if not p.exists():
        pytest.skip(f"{name} not generated")
    return np.load(p)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_speclib_semhat_cubic_bitexact():
    g = _load("fortran_speclib.npz")
    k = 0
    for npt in range(2, 17):
        for fma in (False, True):
            z, w = O.zwgll(npt, fma=fma)
            assert np.array_equal(z, g["zwgll_z"][k:k + npt]), npt
            assert np.array_equal(w, g["zwgll_w"][k:k + npt]), npt
        k += npt
    ka = kb = 0
    for n in range(1, 16):
        np1 = n + 1
        a, b, c, d, z = O.semhat(n, fma=False)
        assert np.array_equal(a, g["semhat_a"][ka:ka + np1 * np1]), n
        assert np.array_equal(c, g["semhat_c"][ka:ka + np1 * np1]), n
        assert np.array_equal(d, g["semhat_d"][ka:ka + np1 * np1]), n
        assert np.array_equal(b, g["semhat_b"][kb:kb + np1]), n
        assert np.array_equal(z, g["semhat_z"][kb:kb + np1]), n
        ka += np1 * np1
        kb += np1
    for npr in range(1, 401):
        assert tuple(O.cubic(npr)) == tuple(g["cubic"][npr - 1]), npr


@pytest.mark.parametrize("path", BOXES, ids=[p.stem for p in BOXES])
def test_box_setup_bitexact(path):
    g = np.load(path)
    nx, ny, nz, lx, _ = (int(v) for v in g["dims"])
    ctx = O.Ctx(nx, ny, nz, lx, mask_mode=0, fma=False)
    glo = O.set_vert_box(lx, ctx.nelt, nx, ny, nz, ctx.lglel)
    assert np.array_equal(glo, g["glo"])
    assert np.array_equal(ctx.setup_g(), g["g"])
    c = ctx.set_multiplicity()
    assert np.array_equal(c, g["c"])
    assert np.array_equal(ctx.set_f(c), g["f"])


@pytest.mark.parametrize("path", BOXES, ids=[p.stem for p in BOXES])
def test_ax_with_reference_mask_bitexact(path):
    """ax twice on a fresh mesh: the first call builds the element-1 mask
    list from its own output, the second applies that list (cg.f:214-258)."""
    g = np.load(path)
    nx, ny, nz, lx, _ = (int(v) for v in g["dims"])
    for fma in (False, True):
        ctx = O.Ctx(nx, ny, nz, lx, mask_mode=0, fma=fma)
        w1 = ctx.ax(g["ax_u"].copy(), g["g"])
        w2 = ctx.ax(g["ax_u"].copy(), g["g"])
        if fma:
            assert _rel(w1, g["ax_w_first"]) < 1e-14
            assert _rel(w2, g["ax_w_second"]) < 1e-14
        else:
            assert np.array_equal(w1, g["ax_w_first"])
            assert np.array_equal(w2, g["ax_w_second"])


def _run_driver_cg(ctx, g, niter):
    c = ctx.set_multiplicity()
    f = ctx.set_f(c)
    gg = ctx.setup_g()
    work = tuple(np.zeros(ctx.n) for _ in range(5))
    first = ctx.cg(f, gg, c, niter, work=work)
    x1, r1, h1 = first["x"].copy(), first["r"].copy(), first["hist"].copy()
    second = ctx.cg(f, gg, c, niter, work=work)
    return x1, r1, h1, second["x"], second["r"], second["hist"]


def _check_history(hist, log, exact):
    """glsc3 values in the reference's order: rnorm^2 at iteration 0, then
    per iteration rtz1, pap, rtr (cg.f:42,52,59,66)."""
    niter = (len(log) - 1) // 3
    assert len(log) == 1 + 3 * niter
    rnorm = np.sqrt(log[0::3])          # iteration 0 and every rtr
    rtz1, pap = log[1::3], log[2::3]
    cmp = (lambda a, b: np.array_equal(a, b)) if exact else \
        (lambda a, b: np.allclose(a, b, rtol=1e-12, atol=0))
    assert cmp(hist[:, 0], rnorm)
    assert cmp(hist[1:, 3], pap)
    assert cmp(hist[1:, 4], rtz1)


@pytest.mark.parametrize("path", BOXES, ids=[p.stem for p in BOXES])
def test_cg_driver_sequence(path):
    g = np.load(path)
    nx, ny, nz, lx, niter = (int(v) for v in g["dims"])
    for fma in (False, True):
        ctx = O.Ctx(nx, ny, nz, lx, mask_mode=0, fma=fma)
        x1, r1, h1, x2, r2, h2 = _run_driver_cg(ctx, g, niter)
        if fma:
            assert _rel(x1, g["x_warmup"]) < 1e-13
            assert _rel(x2, g["x_timed"]) < 1e-13
            _check_history(h1, g["log_warmup"], exact=False)
            _check_history(h2, g["log_timed"], exact=False)
        else:
            assert np.array_equal(x1, g["x_warmup"])
            assert np.array_equal(r1, g["r_warmup"])
            assert np.array_equal(x2, g["x_timed"])
            assert np.array_equal(r2, g["r_timed"])
            _check_history(h1, g["log_warmup"], exact=True)
            _check_history(h2, g["log_timed"], exact=True)
            assert ctx.flops()[1] == float(g["flop_cg"])


def test_c1_configuration():
    """C1: 4^3 elements, lx1=10, the driver's two 100-iteration cg calls."""
    g = _load("fortran_c1_4x4x4_lx10.npz")
    ctx = O.Ctx(4, 4, 4, 10, mask_mode=0, fma=False)   # one thread: sequential glsc3
    x1, r1, h1, x2, r2, h2 = _run_driver_cg(ctx, g, 100)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    assert sha(x1) == str(g["sha_x_warmup"])
    assert sha(x2) == str(g["sha_x_timed"])
    assert sha(r2) == str(g["sha_r_timed"])
    assert np.array_equal(x2[::37], g["x_timed_sample"])
    _check_history(h1, g["log_warmup"], exact=True)
    _check_history(h2, g["log_timed"], exact=True)


def test_hsmg_solve_and_pcg():
    g = _load("fortran_hsmg_2x2x2_lx6.npz")
    nx, ny, nz, lx, niter = (int(v) for v in g["dims"])
    ctx = O.Ctx(nx, ny, nz, lx, mask_mode=0, fma=False)
    assert ctx.h1mg_setup() == 0
    assert ctx.h1mg_levels() == [int(v) for v in g["mg_nx"][:int(g["mg_lmax"])]]
    rhs = g["f"].copy()
    z = ctx.h1mg_solve(rhs)
    assert np.array_equal(rhs, g["rhs_after"])        # h1mg_solve masks rhs in place
    assert _rel(z, g["z"]) < 1e-12
    ctx2 = O.Ctx(nx, ny, nz, lx, mask_mode=0, fma=False)
    assert ctx2.h1mg_setup() == 0
    c = ctx2.set_multiplicity()
    f = ctx2.set_f(c)
    out = ctx2.cg(f, ctx2.setup_g(), c, niter, use_mg=True)
    assert _rel(out["x"], g["pcg_x"]) < 1e-10
    _check_history(out["hist"], g["pcg_log"], exact=False)


def _trace_meshes(z):
    """Per mesh of a driver trace: the nekbone_common values and the
    indices of the calls that follow it up to the next mesh."""
    import json
    calls = json.loads(str(z["calls"]))
    meshes = []
    for k, call in enumerate(calls):
        if call["name"] == "nekbone_mask_reset":      # init_mesh starts a mesh
            meshes.append(dict(calls=[]))
        if call["name"] == "nekbone_common":
            meshes[-1].update(dims=[int(z[f"c{k}_a{j}_in"][0]) for j in range(5)],
                              lglel=z[f"c{k}_a5_in"], dxm1=z[f"c{k}_a6_in"])
        meshes[-1]["calls"].append((k, call["name"]))
    return calls, meshes


@pytest.mark.parametrize("tag", ["plain", "mgrid"])
def test_driver_program_trace_matches_oracle(tag):
    """The boundary calls of driver.f's own program (make_golden_driver.py)
    against the oracle: per mesh, the published dxm1 and the cg inputs (c, f,
    g) are the oracle's set-up, set_multiplicity's gs_op returns the counts,
    and the warm-up and timed cg return the oracle's x and r -- bit for bit
    without the preconditioner, to 1e-12 with hsmg (two eigensolvers)."""
    z = _load(f"driver_trace_{tag}.npz")
    calls, meshes = _trace_meshes(z)
    names = [c["name"] for c in calls]
    # driver.f's order per mesh: init_mesh's reset, proxy_setupds's
    # gs_setup, set_multiplicity's gs_op, the hand-off after proxy_setup,
    # h1mg_setup, set_f's dssum, the two cg calls, gs_free
    per_mesh = ["nekbone_mask_reset", "gs_setup", "gs_op", "nekbone_common",
                "nekbone_set_mask_mode", "nekbone_set_mgrid", "h1mg_setup", "dssum", "cg", "cg",
                "gs_free"]
    assert names == per_mesh * len(meshes)
    mg = tag == "mgrid"
    for m in meshes:
        nelx, nely, nelz, nelt, nx1 = m["dims"]
        assert nelx * nely * nelz == nelt
        ctx = O.Ctx(nelx, nely, nelz, nx1, mask_mode=0, lglel=m["lglel"], fma=False)
        assert np.array_equal(ctx.dxm1(), m["dxm1"])
        if mg:
            assert ctx.h1mg_setup() == 0
        c = ctx.set_multiplicity()
        f = ctx.set_f(c)
        g = ctx.setup_g()
        cg_calls = [k for k, name in m["calls"] if name == "cg"]
        k_op = [k for k, name in m["calls"] if name == "gs_op"][0]
        assert np.array_equal(1.0 / z[f"c{k_op}_a1_out"], c)
        work = tuple(np.zeros(ctx.n) for _ in range(5))
        for k in cg_calls:
            assert int(z[f"c{k}_a8_in"][0]) == ctx.n and int(z[f"c{k}_a9_in"][0]) == 100
            assert np.array_equal(z[f"c{k}_a3_in"], c)
            assert np.array_equal(z[f"c{k}_a1_in"], f)
            assert np.array_equal(z[f"c{k}_a2_in"], g)
            out = ctx.cg(f, g, c, 100, use_mg=mg, work=work)
            if mg:
                assert _rel(out["x"], z[f"c{k}_a0_out"]) < 1e-12
            else:
                assert np.array_equal(out["x"], z[f"c{k}_a0_out"]), k
                assert np.array_equal(out["r"], z[f"c{k}_a4_out"]), k

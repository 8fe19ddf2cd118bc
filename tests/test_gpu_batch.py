"""Batched uneven solves (nb_batch_*): many box problems of different element
counts and lx1 solved by one graph launch of the mixed solver.

Checks, per problem, against the oracle on the same inputs:
  * the set-up is the single-mesh one: g (setup_g form) and c (inverse
    multiplicity) bit-exact with the oracle, f bit-exact with the single-mesh
    nb_rhs_uniform for seed + p;
  * the solution meets the tolerance by the oracle's own residual:
    |f - A x|_C / |f|_C <= 2e-10 (solve tolerance 1e-10; the oracle evaluates
    A x in its own order, which moves the residual by ~1e-16 |A||x|);
  * it agrees with the oracle's FP64 CG solution to 1e-8 relative
    (conditioning of the shifted Laplacian times 1e-10);
  * every instantiated operator shape gives bit-identical iterates (the
    shapes change the launch geometry, not the arithmetic order);
  * converged or zero-right-hand-side problems drop out and the loop ends
    within its cycle bound.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu

BOXES = [(2, 2, 2, 6), (3, 1, 2, 4), (1, 2, 3, 8), (2, 2, 1, 10), (1, 1, 2, 12),
         (3, 2, 2, 6), (1, 1, 1, 4), (2, 1, 1, 8)]


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


class _Dev:
    """A device array seen through __cuda_array_interface__."""

    def __init__(self, ptr, n, typestr="<f8"):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                         "data": (ptr, False), "version": 3}


def _view(torch, ptr, n):
    return torch.as_tensor(_Dev(ptr, n), device="cuda")


def _problem_arrays(torch, b, p):
    x, f, g, c = b.arrays()
    off, n, lx = b.problem(p)
    get = lambda base, k=1: _view(torch, base + 8 * k * off, k * n).cpu().numpy().copy()
    return dict(x=get(x), f=get(f), g=get(g, 6), c=get(c), n=n, lx=lx)


@pytest.fixture(scope="module")
def solved(torch):
    import nekbone_gb300 as nb
    b = nb.Batch(BOXES)
    b.setup(17)
    b.tune(1)
    b.solve(1e-10, 20, 40)
    nb.sync()
    return b


def test_batch_layout(solved):
    b = solved
    assert b.nprob == len(BOXES)
    total = sum(nx * ny * nz * lx ** 3 for nx, ny, nz, lx in BOXES)
    assert b.n == total
    assert b.nlx == len({bx[3] for bx in BOXES})
    # problems are stored by lx1; offsets tile the arrays without overlap
    spans = sorted(b.problem(p)[:2] for p in range(b.nprob))
    pos = 0
    for off, n in spans:
        assert off == pos
        pos += n
    assert pos == total


def test_setup_matches_single_mesh(torch, solved):
    import nekbone_gb300 as nb
    b = solved
    for p, (nx, ny, nz, lx) in enumerate(BOXES):
        a = _problem_arrays(torch, b, p)
        ctx = O.Ctx(nx, ny, nz, lx, mask_mode=1)
        assert np.array_equal(a["g"], ctx.setup_g()), p
        assert np.array_equal(a["c"], ctx.set_multiplicity()), p
        m = nb.DeviceMesh(nx, ny, nz, lx, mask_mode=1)
        cd = torch.from_numpy(a["c"]).cuda()
        fd = torch.empty_like(cd)
        m.rhs_uniform(fd.data_ptr(), cd.data_ptr(), 17 + p)
        assert np.array_equal(fd.cpu().numpy(), a["f"]), p
        m.close()


def test_every_problem_converged_by_oracle_residual(torch, solved):
    b = solved
    for p, (nx, ny, nz, lx) in enumerate(BOXES):
        outer, inner, rr = b.result(p)
        assert rr <= 1e-10, (p, rr)
        assert outer >= 1 and inner == 20 * outer
        a = _problem_arrays(torch, b, p)
        ctx = O.Ctx(nx, ny, nz, lx, mask_mode=1)
        r = a["f"] - ctx.ax(a["x"], a["g"])
        rel = np.sqrt(np.sum(r * a["c"] * r)) / np.sqrt(np.sum(a["f"] * a["c"] * a["f"]))
        assert rel <= 2e-10, (p, rel)
    assert 1 <= solved.cycles() <= 41


def test_solution_matches_oracle_cg(torch, solved):
    b = solved
    for p in (0, 3, 4):
        nx, ny, nz, lx = BOXES[p]
        a = _problem_arrays(torch, b, p)
        ctx = O.Ctx(nx, ny, nz, lx, mask_mode=1)
        res = ctx.cg(a["f"].copy(), a["g"], a["c"], 300)
        xo = res["x"]
        assert np.max(np.abs(a["x"] - xo)) <= 1e-8 * np.max(np.abs(xo)), p


def test_shapes_bit_identical(torch):
    import nekbone_gb300 as nb
    boxes = [(2, 2, 1, 4), (2, 1, 2, 6), (1, 2, 2, 8), (2, 1, 1, 10), (1, 1, 2, 12)]
    b = nb.Batch(boxes)
    b.setup(3)
    ref = None
    shapes = {4: [(4, 1, 4), (8, 0, 8), (16, 1, 4)], 6: [(2, 1, 2), (4, 0, 4), (8, 1, 2)],
              8: [(1, 1, 1), (2, 0, 2), (4, 1, 1)], 10: [(1, 1, 1), (2, 0, 2), (4, 1, 1)],
              12: [(1, 1, 1), (2, 0, 2), (4, 1, 1)]}
    for k in range(3):
        for lx, opts in shapes.items():
            b.set_tuning(lx, *opts[k])
        b.solve(1e-10, 20, 40)
        nb.sync()
        x = _view(torch, b.arrays()[0], b.n).cpu().numpy().copy()
        res = [b.result(p) for p in range(len(boxes))]
        if ref is None:
            ref = (x, res)
        else:
            assert np.array_equal(x, ref[0]), k
            assert res == ref[1], k
    b.close()


@pytest.mark.parametrize("itol,inner", [(0.0, 20), (1e-4, 30), (0.0, 7)])
def test_inner_forms_bit_identical(torch, itol, inner):
    """The inner CG's streamlined forms against the plain one: c formed in
    closed form (verified at setup as every problem's inverse multiplicity)
    or read, and the directions in two buffers with x updated once per pair
    of iterations (problems that stop their inner CG on the first of a pair
    get the deferred update before the defect; an odd inner count leaves the
    last iteration unpaired) or one buffer.  Bit-identical solutions,
    per-problem results and cycle counts."""
    import nekbone_gb300 as nb
    b = nb.Batch(BOXES)
    b.setup(23)
    b.set_inner_tol(itol)
    got = []
    try:
        for closed, paired in ((True, True), (False, True), (True, False), (False, False),
                               (True, True)):
            nb.set_mixed_closed_multiplicity(closed)
            nb.set_paired_update(paired)
            b.solve(1e-10, inner, 40)
            nb.sync()
            x = _view(torch, b.arrays()[0], b.n).cpu().numpy().copy()
            got.append((x, [b.result(p) for p in range(b.nprob)], b.cycles()))
    finally:
        nb.set_mixed_closed_multiplicity(True)
        nb.set_paired_update(True)
    for k, (x, res, cyc) in enumerate(got[1:]):
        assert np.array_equal(x, got[0][0]), k
        assert res == got[0][1] and cyc == got[0][2], k
    b.close()


def test_cycle_bound_and_zero_rhs(torch):
    import nekbone_gb300 as nb
    boxes = [(2, 2, 2, 6), (1, 1, 1, 8), (2, 1, 1, 4)]
    b = nb.Batch(boxes)
    b.setup(5)
    # one cycle only: every problem stops after it, above the tolerance
    b.solve(1e-10, 5, 1)
    nb.sync()
    assert b.cycles() == 1
    for p in range(3):
        outer, inner, rr = b.result(p)
        assert (outer, inner) == (1, 5) and rr > 1e-10
    # problem 1 with f = 0 is inactive from the start; the others converge
    f = _view(torch, b.arrays()[1], b.n)
    off, n, _ = b.problem(1)
    f[off:off + n] = 0.0
    torch.cuda.synchronize()
    b.solve(1e-10, 20, 40)
    nb.sync()
    assert b.result(1) == (0, 0, 0.0)
    x = _view(torch, b.arrays()[0], b.n).cpu().numpy()
    assert np.all(x[off:off + n] == 0.0)
    for p in (0, 2):
        assert b.result(p)[2] <= 1e-10
    b.close()


def test_host_copies_round_trip(torch):
    import nekbone_gb300 as nb
    boxes = [(2, 1, 1, 6), (1, 2, 1, 8)]
    b = nb.Batch(boxes)
    b.setup(9)
    fdev = _view(torch, b.arrays()[1], b.n).cpu()
    fh = torch.empty(b.n, dtype=torch.float64).pin_memory()
    fh.copy_(fdev * 2.0)
    b.rhs_in(fh.data_ptr())
    b.solve(1e-10, 20, 40)
    xh = torch.empty(b.n, dtype=torch.float64).pin_memory()
    b.x_out(xh.data_ptr())
    nb.sync()
    xd = _view(torch, b.arrays()[0], b.n).cpu()
    assert torch.equal(xh, xd)
    assert torch.equal(_view(torch, b.arrays()[1], b.n).cpu(), fh)
    for p in range(2):
        assert b.result(p)[2] <= 1e-10
    b.close()


def test_even_odd_forms_agree(torch):
    """The even-odd forms (one line per thread; FP32 metric by bulk copy)
    sum in a different order: same tolerance met, solutions within 1e-8."""
    import nekbone_gb300 as nb
    boxes = [(2, 2, 1, 4), (2, 1, 2, 6), (1, 2, 2, 8), (2, 1, 1, 10), (1, 1, 2, 12)]
    b = nb.Batch(boxes)
    b.setup(3)
    xs = []
    for eo in (False, True):
        for lx in (4, 6, 8, 10, 12):
            if eo:
                b.set_tuning(lx, 1, 2, 0)
            else:
                b.set_tuning(lx, 4 if lx == 4 else (2 if lx == 6 else 1), 1,
                             4 if lx == 4 else (2 if lx == 6 else 1))
        b.solve(1e-10, 20, 40)
        nb.sync()
        xs.append(_view(torch, b.arrays()[0], b.n).cpu().numpy().copy())
        for p in range(len(boxes)):
            assert b.result(p)[2] <= 1e-10
    assert np.max(np.abs(xs[0] - xs[1])) <= 1e-8 * np.max(np.abs(xs[0]))
    b.close()


def test_inner_tolerance_stops_each_problem(torch):
    """With an inner tolerance each problem's FP32 CG ends its cycle once its
    residual fell by itol (at most inner_iters): every problem still meets
    the outer tolerance by the oracle's residual, and the small problems
    stop early."""
    import nekbone_gb300 as nb
    b = nb.Batch(BOXES)
    b.setup(17)
    b.tune(1)
    b.set_inner_tol(1e-4)
    b.solve(1e-10, 60, 40)
    nb.sync()
    early = 0
    for p, (nx, ny, nz, lx) in enumerate(BOXES):
        outer, inner, rr = b.result(p)
        assert rr <= 1e-10, (p, rr)
        assert 1 <= outer and outer <= inner <= 60 * outer
        early += inner < 60 * outer
        a = _problem_arrays(torch, b, p)
        ctx = O.Ctx(nx, ny, nz, lx, mask_mode=1)
        r = a["f"] - ctx.ax(a["x"], a["g"])
        rel = np.sqrt(np.sum(r * a["c"] * r)) / np.sqrt(np.sum(a["f"] * a["c"] * a["f"]))
        assert rel <= 2e-10, (p, rel)
    assert early >= 1
    # back to the fixed count: every cycle runs inner_iters again
    b.set_inner_tol(0.0)
    b.solve(1e-10, 20, 40)
    nb.sync()
    for p in range(len(BOXES)):
        outer, inner, rr = b.result(p)
        assert inner == 20 * outer and rr <= 1e-10
    b.close()


def test_phase_timing_runs_the_same_solve(torch):
    """nb_batch_time_phases launches the graph solve's kernels one cycle at a
    time with events between them: bit-identical x and per-problem results,
    the same cycle count, and a positive time for every phase that ran."""
    import nekbone_gb300 as nb
    b = nb.Batch(BOXES)
    b.setup(17)
    b.tune(1)
    b.set_inner_tol(1e-4)
    b.solve(1e-10, 30, 40)
    nb.sync()
    x_graph = _view(torch, b.arrays()[0], b.n).cpu().numpy().copy()
    res_graph = [b.result(p) for p in range(b.nprob)]
    cyc_graph = b.cycles()
    _view(torch, b.arrays()[0], b.n).fill_(float("nan"))
    torch.cuda.synchronize()
    ms, cyc = b.time_phases(1e-10, 30, 40)
    x = _view(torch, b.arrays()[0], b.n).cpu().numpy()
    assert cyc == cyc_graph == b.cycles() and cyc >= 2
    assert np.array_equal(x, x_graph)
    assert [b.result(p) for p in range(b.nprob)] == res_graph
    assert set(ms) == set(nb.Batch.PHASES)
    assert all(v > 0.0 for v in ms.values()), ms
    print("batched phases (ms):", {k: round(v, 4) for k, v in ms.items()})
    b.close()


def test_fixed_point_defect_operator(torch):
    """The FP64 defect in the fixed-point form (epb64 = -1: x += |r| e, then
    the fixed-point element operator on the integer pipes) against the
    even-odd FP64-pipe form: both meet the tolerance by the oracle's own
    residual, and the solutions agree to 1e-8 (the two operators agree to
    rounding, ~1e-15 per apply)."""
    import nekbone_gb300 as nb
    b = nb.Batch(BOXES)
    b.setup(17)
    xs = []
    for epb64 in (-1, 0):
        for lx in sorted({bx[3] for bx in BOXES}):
            t = b.tuning(lx)
            b.set_tuning(lx, t["epb32"], t["rd32"], epb64)
            assert b.tuning(lx)["epb64"] == epb64
        b.solve(1e-10, 20, 40)
        nb.sync()
        xs.append(_view(torch, b.arrays()[0], b.n).cpu().numpy().copy())
        for p, (nx, ny, nz, lx) in enumerate(BOXES):
            a = _problem_arrays(torch, b, p)
            ctx = O.Ctx(nx, ny, nz, lx, mask_mode=1)
            r = a["f"] - ctx.ax(a["x"], a["g"])
            rel = np.sqrt(np.sum(r * a["c"] * r)) / np.sqrt(np.sum(a["f"] * a["c"] * a["f"]))
            assert rel <= 2e-10, (epb64, p, rel)
    assert np.max(np.abs(xs[0] - xs[1])) <= 1e-8 * np.max(np.abs(xs[1]))
    b.close()

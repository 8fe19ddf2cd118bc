"""CPU tests of the oracle: pinned against the reference's own jl library
(golden vectors in tests/golden/, generated by tests/golden/make_golden.py from
jl compiled out of the reference sources), the known answers of jl's own test
programs, closed forms of the GLL rule, and mathematical identities of the
operator, CG and multigrid restatements."""
from __future__ import annotations

import glob
import math
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O

GOLDEN = sorted(glob.glob(str(Path(__file__).parent / "golden" / "gs_*.npz")))
DT = {1: np.float64, 2: np.float32, 3: np.int32, 4: np.int64}


@pytest.mark.parametrize("path", GOLDEN, ids=[Path(p).stem for p in GOLDEN])
def test_gs_maps_match_jl(path):
    g = np.load(path)
    h = O.Gs(g["ids"])
    m = h.maps()
    for w in range(3):
        assert np.array_equal(m[w], g[f"map{w}"]), f"map{w}"


@pytest.mark.parametrize("path", GOLDEN, ids=[Path(p).stem for p in GOLDEN])
def test_gs_op_matches_jl(path):
    g = np.load(path)
    h = O.Gs(g["ids"])
    for dom in (1, 2, 3, 4):
        for op in (1, 2, 3, 4):
            for tr in (0, 1):
                u = g[f"in_{dom}_{op}_{tr}"].copy()
                if len(u):
                    h.op(u, dom, op, tr)
                ref = g[f"out_{dom}_{op}_{tr}"]
                assert u.dtype == ref.dtype
                assert np.array_equal(u.view(np.uint8), ref.view(np.uint8)), (dom, op, tr)


def test_gs_known_answers():
    """jl/gs_test.c at one process prints 0 3 3 3 3 then 1 1 4 4 4."""
    h = O.Gs(np.array([-11, -1, 1, 1, 1]))
    v = np.ones(5)
    h.op(v, 1, 1, 0)
    assert v.tolist() == [0, 3, 3, 3, 3]
    v = np.ones(5)
    h.op(v, 1, 1, 1)
    assert v.tolist() == [1, 1, 4, 4, 4]


def test_gs_fuzz_against_reference_library():
    ref = Path(O.ROOT / "oracle" / "_ref" / "libjl_ref.so")
    if not ref.exists():
        pytest.skip("reference jl library not built here (needs the reference checkout)")
    import ctypes as C
    jl = C.CDLL(str(ref))
    jl.jlp_gs_setup.restype = C.c_void_p
    rng = np.random.default_rng(11)
    for trial in range(20):
        n = int(rng.integers(1, 3000))
        ids = rng.integers(-int(rng.integers(1, 400)), 400, size=n).astype(np.int64)
        h = O.Gs(ids)
        hj = jl.jlp_gs_setup(O._p(ids), C.c_int(n))
        mine = h.maps()
        for w in range(3):
            ln = jl.jlp_map_len(C.c_void_p(hj), C.c_int(w))
            m = np.zeros(ln, dtype=np.uint32)
            jl.jlp_map_copy(C.c_void_p(hj), C.c_int(w), O._p(m))
            assert np.array_equal(m, mine[w])
        u = rng.standard_normal(n)
        v = u.copy()
        h.op(u, 1, 1, 0)
        jl.jlp_gs_op(C.c_void_p(hj), O._p(v), C.c_int(1), C.c_int(1), C.c_int(0))
        assert np.array_equal(u, v)
        jl.jlp_gs_free(C.c_void_p(hj))


# ------------------------------------------------------------------ GLL --
def test_gll_closed_forms():
    z, w = O.zwgll(2)
    assert z.tolist() == [-1, 1] and np.allclose(w, [1, 1], atol=1e-15)
    z, w = O.zwgll(3)
    assert np.allclose(z, [-1, 0, 1], atol=1e-15) and np.allclose(w, [1 / 3, 4 / 3, 1 / 3], atol=1e-15)
    z, w = O.zwgll(4)
    s = 1 / math.sqrt(5)
    assert np.allclose(z, [-1, -s, s, 1], atol=1e-15)
    assert np.allclose(w, [1 / 6, 5 / 6, 5 / 6, 1 / 6], atol=1e-15)
    z, w = O.zwgll(5)
    t = math.sqrt(3 / 7)
    assert np.allclose(z, [-1, -t, 0, t, 1], atol=1e-15)
    assert np.allclose(w, [0.1, 49 / 90, 32 / 45, 49 / 90, 0.1], atol=1e-15)


@pytest.mark.parametrize("np_", [6, 8, 10, 12, 16])
def test_gll_legendre_identities(np_):
    z, w = O.zwgll(np_)
    n = np_ - 1
    c = np.zeros(n + 1)
    c[-1] = 1
    pn = np.polynomial.legendre.legval(z, c)
    dpn = np.polynomial.legendre.legval(z, np.polynomial.legendre.legder(c))
    assert np.max(np.abs(dpn[1:-1])) < 1e-11          # interior nodes: P_N'(z) = 0
    assert np.allclose(w, 2 / (n * (n + 1) * pn ** 2), rtol=1e-13)
    assert np.allclose(z, -z[::-1], atol=1e-15)
    for k in range(2 * n - 1):                        # exact for degree 2N-1
        assert abs(np.dot(w, z ** k) - (2 / (k + 1) if k % 2 == 0 else 0)) < 1e-13


@pytest.mark.parametrize("n", [1, 3, 7, 9, 11, 15])
def test_semhat_derivative_exact(n):
    a, b, c, d, z = O.semhat(n)
    m = n + 1
    D = d.reshape(m, m, order="F")
    for k in range(m):
        assert np.allclose(D @ z ** k, k * z ** (k - 1) if k else 0 * z, atol=1e-10 * max(1, k) * m)
    A = a.reshape(m, m, order="F")
    assert np.allclose(A, A.T, atol=1e-12)
    assert np.allclose(A @ np.ones(m), 0, atol=1e-11)
    assert np.allclose(A, D.T @ np.diag(b) @ D, atol=1e-11)


def test_cubic():
    assert O.cubic(64) == (4, 4, 4)
    assert O.cubic(32768) == (32, 32, 32)
    assert O.cubic(50) == (5, 5, 2)
    assert O.cubic(7) == (7, 1, 1)
    assert O.cubic(12) == (3, 2, 2)


def test_set_vert_box_numbering():
    nelx, nely, nelz, nx = 3, 2, 2, 4
    nelt = nelx * nely * nelz
    g = O.set_vert_box(nx, nelt, nelx, nely, nelz, np.arange(1, nelt + 1))
    nn = nx - 1
    assert g.min() == 1 and g.max() == (nn * nelx + 1) * (nn * nely + 1) * (nn * nelz + 1)
    assert len(np.unique(g)) == g.max()
    _, cnt = np.unique(g, return_counts=True)
    assert set(cnt.tolist()) <= {1, 2, 4, 8}


# ------------------------------------------------------------------- cg.f --
def _continuous(ctx, rng):
    """a random field that is single-valued at shared points"""
    glo = O.set_vert_box(ctx.nx1, ctx.nelt, ctx.nelx, ctx.nely, ctx.nelz, ctx.lglel)
    vals = rng.standard_normal(glo.max() + 1)
    return vals[glo]


def test_ax_symmetric_and_shift():
    ctx = O.Ctx(3, 2, 2, 5, mask_mode=1)
    g = ctx.setup_g()
    c = ctx.set_multiplicity()
    rng = np.random.default_rng(0)
    u, v = _continuous(ctx, rng), _continuous(ctx, rng)
    ctx.maskit(u)
    ctx.maskit(v)
    au, av = ctx.ax(u, g), ctx.ax(v, g)
    L = O.load()
    import ctypes as C
    a = L.orc_glsc3(O._p(v), O._p(c), O._p(au), C.c_int(ctx.n))
    b = L.orc_glsc3(O._p(u), O._p(c), O._p(av), C.c_int(ctx.n))
    assert abs(a - b) < 1e-12 * max(abs(a), 1)
    # constant field: A_L 1 = 0, so A 1 = 0.1 (before masking)
    one = np.ones(ctx.n)
    w = ctx.ax_local(one, g)
    assert np.max(np.abs(w)) < 1e-12


def test_ax_linear_field_interior_zero():
    """The weak Laplacian of a linear field vanishes at interior nodes."""
    nelx, nely, nelz, nx = 3, 3, 3, 6
    ctx = O.Ctx(nelx, nely, nelz, nx, mask_mode=1)
    g = ctx.setup_g()
    z = O.zwgll(nx)[0]
    u = np.zeros(ctx.n)
    w_unmasked = np.zeros(ctx.n)
    p = 0
    for ez in range(nelz):
        for ey in range(nely):
            for ex in range(nelx):
                for k in range(nx):
                    for j in range(nx):
                        for i in range(nx):
                            X, Y, Zc = 2 * ex + z[i], 2 * ey + z[j], 2 * ez + z[k]
                            u[p] = 0.3 * X - 1.1 * Y + 0.7 * Zc + 2.0
                            p += 1
    w_unmasked = ctx.ax_local(u, g)
    ctx.dssum(w_unmasked)
    c = ctx.set_multiplicity()
    mask = np.ones(ctx.n)
    ctx.maskit(mask)
    interior = mask == 1
    assert np.max(np.abs(w_unmasked[interior])) < 1e-10


def test_maskit_reference_quirk():
    """First call zeroes every element's outer faces and records only element
    1's zero indices (cg.f:236-254); later calls zero only those."""
    ctx = O.Ctx(3, 1, 1, 4, mask_mode=0)
    w = np.ones(ctx.n)
    ctx.maskit(w)
    nxyz = 64
    # element 2 (the middle one) has interior faces in x but outer y/z faces
    assert np.count_nonzero(w[nxyz:2 * nxyz] == 0) > 0
    w2 = np.ones(ctx.n)
    ctx.maskit(w2)
    assert np.all(w2[nxyz:] == 1)              # only element 1 is masked now
    assert np.array_equal(w2[:nxyz] == 0, w[:nxyz] == 0)


def test_cg_converges_and_residual_consistent():
    ctx = O.Ctx(4, 4, 4, 6, mask_mode=1)
    g = ctx.setup_g()
    c = ctx.set_multiplicity()
    f = ctx.set_f(c)
    ctx.maskit(f)
    out = ctx.cg(f, g, c, 100)
    h = out["hist"]
    assert out["iter"] == 101
    assert h[-1, 0] < 1e-6 * h[0, 0]
    r = f - ctx.ax(out["x"], g)
    assert np.max(np.abs(r - out["r"])) < 1e-9 * np.max(np.abs(f))


def test_flop_counters_wrap_like_int32():
    ctx = O.Ctx(2, 2, 2, 4, mask_mode=1)
    g = ctx.setup_g()
    c = ctx.set_multiplicity()
    f = ctx.set_f(c)
    ctx.cg(f, g, c, 3)
    fa, fc = ctx.flops()
    nxyz = 64
    assert fa == 3 * (19 * nxyz + 12 * 4 * nxyz) * 8
    assert fc == 4 * 15 * ctx.n


# ---------------------------------------------------------------- hsmg.f --
def test_generalev_against_scipy():
    sl = pytest.importorskip("scipy.linalg")
    import ctypes as C
    rng = np.random.default_rng(3)
    L = O.load()
    for n in (4, 7, 12):
        M = rng.standard_normal((n, n))
        A = M + M.T
        R = rng.standard_normal((n, n))
        B = R @ R.T + n * np.eye(n)
        a = np.asfortranarray(A).ravel(order="F").copy()
        b = np.asfortranarray(B).ravel(order="F").copy()
        lam = np.zeros(n)
        assert L.orc_generalev(O._p(a), O._p(b), O._p(lam), C.c_int(n)) == 0
        X = a.reshape(n, n, order="F")
        ref = sl.eigh(A, B, eigvals_only=True)
        assert np.allclose(lam, ref, rtol=1e-12, atol=1e-12)
        assert np.allclose(X.T @ B @ X, np.eye(n), atol=1e-11)
        assert np.allclose(A @ X, B @ X @ np.diag(lam), atol=1e-10)


def test_h1mg_reference_levels():
    for nx1, want in ((4, [1, 3]), (5, [1, 2, 4]), (8, [1, 3, 7]), (10, [1, 3, 9])):
        ctx = O.Ctx(2, 2, 2, nx1, mask_mode=1)
        assert ctx.h1mg_setup() == 0
        assert ctx.h1mg_levels() == want


def test_h1mg_linear_and_accelerates_cg():
    ctx = O.Ctx(3, 3, 3, 8, mask_mode=1)
    assert ctx.h1mg_setup() == 0
    g = ctx.setup_g()
    c = ctx.set_multiplicity()
    rng = np.random.default_rng(5)
    r1, r2 = _continuous(ctx, rng), _continuous(ctx, rng)
    ctx.maskit(r1)
    ctx.maskit(r2)
    z1 = ctx.h1mg_solve(r1.copy())
    z2 = ctx.h1mg_solve(r2.copy())
    z12 = ctx.h1mg_solve((2 * r1 - 3 * r2).copy())
    assert np.allclose(z12, 2 * z1 - 3 * z2, atol=1e-10 * np.max(np.abs(z12)))
    f = ctx.set_f(c)
    ctx.maskit(f)
    plain = ctx.cg(f, g, c, 30)["hist"][:, 0]
    pre = ctx.cg(f, g, c, 30, use_mg=True)["hist"][:, 0]
    assert pre[-1] / pre[0] < 0.1 * plain[-1] / plain[0]

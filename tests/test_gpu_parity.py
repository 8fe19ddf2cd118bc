"""GPU parity tests: the CUDA path, called through the C ABI, against the
oracle on the same inputs.

Tolerances: integer maps and gather-scatter results are bit-exact; the
element operator (ax, local_grad3, mxm) is bit-exact against the oracle's fma
variant because both evaluate every contraction as the same left-to-right fma
chain; quantities that go through a dot product (glsc3, and so the CG
iterates) differ only by the summation order of the reduction and must agree
to 1e-12 relative, also through the multigrid preconditioner (its FDM
eigenvectors come from two separately compiled eigensolvers, whose results
agree to ~1e-15).
"""
from __future__ import annotations

import glob
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(str(Path(__file__).parent / "golden" / "gs_*.npz")))


@pytest.fixture(scope="module")
def nb():
    import nekbone_gb300 as m
    return m


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# ------------------------------------------------------------ gather-scatter --
@pytest.mark.parametrize("path", GOLDEN, ids=[Path(p).stem for p in GOLDEN])
def test_gs_op_golden(nb, path):
    g = np.load(path)
    if len(g["ids"]) == 0:
        h = nb.gs_setup(g["ids"])
        nb.gs_free(h)
        return
    h = nb.gs_setup(g["ids"])
    for dom in (1, 2, 3, 4):
        for op in (1, 2, 3, 4):
            for tr in (0, 1):
                u = g[f"in_{dom}_{op}_{tr}"].copy()
                nb.gs_op(h, u, op, tr)
                ref = g[f"out_{dom}_{op}_{tr}"]
                assert np.array_equal(u.view(np.uint8), ref.view(np.uint8)), (dom, op, tr)
    nb.gs_free(h)


@pytest.mark.parametrize("dims", [(4, 4, 4, 10), (3, 2, 5, 7), (1, 1, 1, 3), (6, 1, 1, 2)])
def test_dssum_box_bitexact(nb, dims):
    nelx, nely, nelz, nx = dims
    mesh = nb.Nekbone(nelx, nely, nelz, nx, mask_mode=1)
    ctx = O.Ctx(nelx, nely, nelz, nx, mask_mode=1)
    rng = np.random.default_rng(1)
    u = rng.standard_normal(mesh.n)
    v = u.copy()
    mesh.dssum(u)
    ctx.dssum(v)
    assert np.array_equal(u, v)
    assert np.array_equal(mesh.set_multiplicity(), ctx.set_multiplicity())


def test_gs_invalid_handle_and_params(nb):
    with pytest.raises(nb.NekboneError):
        nb.gs_op(999, np.zeros(4))
    h = nb.gs_setup(np.array([1, 1, 2]))
    nb.gs_free(h)
    with pytest.raises(nb.NekboneError):
        nb.gs_op(h, np.zeros(3))          # freed handles stay invalid
    with pytest.raises(nb.NekboneError):
        nb.gs_op(nb.gs_setup(np.array([1, 1])), np.zeros(2), op=5)


# ----------------------------------------------------------------- kernels --
@pytest.mark.parametrize("shape", [(12, 12, 144), (10, 10, 100), (144, 12, 12), (5, 30, 7), (3, 1, 4)])
def test_mxm_bitexact(nb, shape):
    n1, n2, n3 = shape
    rng = np.random.default_rng(2)
    a, b = rng.standard_normal(n1 * n2), rng.standard_normal(n2 * n3)
    assert np.array_equal(nb.mxm(a, n1, b, n2, n3), O.mxm(a, n1, b, n2, n3, fma=True))


@pytest.mark.parametrize("n", [1, 4, 9, 11, 15])
def test_local_grad3_bitexact(nb, n):
    rng = np.random.default_rng(3)
    m = n + 1
    u = rng.standard_normal(m ** 3)
    D = rng.standard_normal(m * m)
    Dt = rng.standard_normal(m * m)
    L = O.load(True)
    ref = [np.zeros(m ** 3) for _ in range(3)]
    import ctypes as C
    L.orc_local_grad3(*(O._p(x) for x in ref), O._p(u), C.c_int(n), O._p(D), O._p(Dt))
    got = nb.local_grad3(u, n, D, Dt)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    ur, us, ut = ref
    uo, wo = np.zeros(m ** 3), np.zeros(m ** 3)
    L.orc_local_grad3_t(O._p(uo), O._p(ur), O._p(us), O._p(ut), C.c_int(n), O._p(D), O._p(Dt), O._p(wo))
    ug, wg = nb.local_grad3_t(ur, us, ut, n, D, Dt)
    assert np.array_equal(ug, uo) and np.array_equal(wg, wo)


@pytest.mark.parametrize("nx", [2, 3, 6, 8, 10, 12, 16])
def test_ax_e_bitexact(nb, nx):
    mesh = nb.Nekbone(1, 1, 1, nx, mask_mode=1)
    ctx = O.Ctx(1, 1, 1, nx, mask_mode=1)
    rng = np.random.default_rng(4)
    u = rng.standard_normal(nx ** 3)
    g = rng.standard_normal(6 * nx ** 3)
    w = mesh.ax_e(u, g)
    wo = np.zeros(nx ** 3)
    ctx.L.orc_ax_e(ctx.hv, O._p(wo), O._p(u), O._p(g))
    assert np.array_equal(w, wo)


@pytest.mark.parametrize("dims", [(4, 4, 4, 10), (2, 3, 2, 12), (3, 3, 1, 5), (1, 1, 2, 16)])
@pytest.mark.parametrize("mask_mode", [0, 1])
def test_ax_bitexact(nb, dims, mask_mode):
    nelx, nely, nelz, nx = dims
    mesh = nb.Nekbone(nelx, nely, nelz, nx, mask_mode=mask_mode)
    ctx = O.Ctx(nelx, nely, nelz, nx, mask_mode=mask_mode)
    rng = np.random.default_rng(5)
    g = rng.standard_normal(6 * mesh.n)         # a general (deformed) metric
    nb.Nekbone.set_order(0)                     # the reference's summation order
    try:
        for _ in range(2):                     # first call builds the mask list
            u = rng.standard_normal(mesh.n)
            assert np.array_equal(mesh.ax(u, g), ctx.ax(u, g))
        # the even-odd order agrees to rounding
        nb.Nekbone.set_order(1)
        u = rng.standard_normal(mesh.n)
        ref = ctx.ax(u, g)
        assert rel(mesh.ax(u, g), ref) < 1e-13
    finally:
        nb.Nekbone.set_order(nb.DEFAULT_ORDER)


def test_blas1(nb):
    rng = np.random.default_rng(6)
    n = 100003
    a, b, m = rng.standard_normal(n), rng.standard_normal(n), rng.random(n)
    assert abs(nb.glsc3(a, b, m) - O.load().orc_glsc3(O._p(a), O._p(b), O._p(m), n)) < 1e-12 * np.sum(np.abs(a * b * m))
    x = a.copy()
    nb.add2s1(x, b, 0.37)
    y = a.copy()
    nb.add2s2(y, b, -1.25)
    L = O.load(True)
    yo = a.copy()
    import ctypes as C
    L.orc_add2s2(O._p(yo), O._p(b), C.c_double(-1.25), C.c_int(n))
    assert np.array_equal(y, yo)
    xo = a.copy()
    L.orc_add2s1(O._p(xo), O._p(b), C.c_double(0.37), C.c_int(n))
    assert np.array_equal(x, xo)


# ---------------------------------------------------------------------- cg --
@pytest.mark.parametrize("mask_mode", [0, 1])
def test_cg_c1_matches_oracle(nb, mask_mode):
    """Config 1: 4x4x4 elements, lx1=10, 100 iterations, warm-up + timed call
    as driver.f:54-59 makes them (the second call sees the mask list)."""
    mesh = nb.Nekbone(4, 4, 4, 10, mask_mode=mask_mode)
    ctx = O.Ctx(4, 4, 4, 10, mask_mode=mask_mode)
    c = mesh.set_multiplicity()
    g = mesh.setup_g()
    f = mesh.set_f(c)
    assert np.array_equal(c, ctx.set_multiplicity())
    assert np.array_equal(g, ctx.setup_g())
    assert np.array_equal(f, ctx.set_f(c))
    mesh.mask_reset()
    nb.Nekbone.set_flops(0.0, 0.0)
    work = tuple(np.zeros(mesh.n) for _ in range(5))
    owork = tuple(np.zeros(mesh.n) for _ in range(5))
    for call in range(2):
        x, r, w, p, z, fc = mesh.cg(f, g, c, 100, 0.0, work)
        o = ctx.cg(f, g, c, 100, work=owork)
        # r, z and p end ~1e-10 below f (they decay with the residual), so
        # they are compared on f's scale; x is compared on its own scale
        scale = np.max(np.abs(f))
        assert rel(x, o["x"]) < 1e-12, call
        for name, a, b in (("r", r, o["r"]), ("p", p, o["p"]), ("z", z, o["z"]),
                           ("w", w, o["w"])):
            assert np.max(np.abs(a - b)) < 1e-12 * scale, (call, name)
    assert fc == 101 * 15 * mesh.n


@pytest.mark.parametrize("mask_mode", [0, 1])
@pytest.mark.parametrize("niter", [0, 1, 2])
def test_cg_few_iterations_match_oracle(nb, mask_mode, niter):
    """The drop-in cg with 0, 1 and 2 iterations: x, r, w, p (and z once an
    iteration ran) and the flop count (the reference counts niter + 1
    iterations, cg.f:81) as the oracle gives them."""
    mesh = nb.Nekbone(2, 3, 2, 6, mask_mode=mask_mode)
    ctx = O.Ctx(2, 3, 2, 6, mask_mode=mask_mode)
    c = mesh.set_multiplicity()
    g = mesh.setup_g()
    f = mesh.set_f(c)
    mesh.mask_reset()
    nb.Nekbone.set_flops(0.0, 0.0)
    work = tuple(np.zeros(mesh.n) for _ in range(5))
    owork = tuple(np.zeros(mesh.n) for _ in range(5))
    x, r, w, p, z, fc = mesh.cg(f, g, c, niter, 0.0, work)
    o = ctx.cg(f, g, c, niter, work=owork)
    scale = np.max(np.abs(f))
    assert np.max(np.abs(x - o["x"])) <= 1e-13 * max(np.max(np.abs(o["x"])), scale)
    pairs = [("r", r, o["r"]), ("w", w, o["w"]), ("p", p, o["p"])]
    if niter > 0:
        pairs.append(("z", z, o["z"]))
    for name, a, b in pairs:
        assert np.max(np.abs(a - b)) <= 1e-13 * scale, name
    assert fc == (niter + 1) * 15 * mesh.n


@pytest.mark.parametrize("mask_mode", [0, 1])
@pytest.mark.parametrize("dims", [(1, 1, 1, 5), (2, 1, 1, 4), (1, 1, 3, 6)])
def test_cg_smallest_meshes_match_oracle(nb, mask_mode, dims):
    """One element, and a row of two or three: the boundary groups are all
    pairs or singletons (the domain faces), and the drop-in cg still matches
    the oracle."""
    mesh = nb.Nekbone(*dims, mask_mode=mask_mode)
    ctx = O.Ctx(*dims, mask_mode=mask_mode)
    c = mesh.set_multiplicity()
    g = mesh.setup_g()
    f = mesh.set_f(c)
    assert np.array_equal(c, ctx.set_multiplicity())
    mesh.mask_reset()
    work = tuple(np.zeros(mesh.n) for _ in range(5))
    owork = tuple(np.zeros(mesh.n) for _ in range(5))
    for call in range(2):
        x, r, w, p, z, fc = mesh.cg(f, g, c, 10, 0.0, work)
        o = ctx.cg(f, g, c, 10, work=owork)
        scale = np.max(np.abs(f))
        assert np.max(np.abs(x - o["x"])) <= 1e-12 * max(np.max(np.abs(o["x"])), scale), call
        for name, a, b in (("r", r, o["r"]), ("w", w, o["w"]), ("p", p, o["p"])):
            assert np.max(np.abs(a - b)) <= 1e-12 * scale, (call, name)


def test_cg_seeded_rhs_device_api(nb):
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(4, 4, 4, 10, mask_mode=1)
    ctx = O.Ctx(4, 4, 4, 10, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    m.setup_g(g.data_ptr())
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 1234)
    torch.cuda.synchronize()
    vs = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(5)]
    hist = m.cg(*(t.data_ptr() for t in (vs[0], f, g, c, vs[1], vs[2], vs[3], vs[4])), 100, hist=True)
    fh, gh, ch = f.cpu().numpy(), g.cpu().numpy(), c.cpu().numpy()
    assert np.array_equal(gh, ctx.setup_g()) and np.array_equal(ch, ctx.set_multiplicity())
    assert np.all(np.abs(fh) <= 1.0) and np.abs(fh).max() > 0.5
    o = ctx.cg(fh, gh, ch, 100)
    assert rel(vs[0].cpu().numpy(), o["x"]) < 1e-12
    assert np.allclose(hist[:, 0], o["hist"][:, 0], rtol=1e-10, atol=0)
    # the unfused path gives the same iterates
    vs2 = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(5)]
    m.cg(*(t.data_ptr() for t in (vs2[0], f, g, c, vs2[1], vs2[2], vs2[3], vs2[4])), 100, flags=1)
    assert rel(vs2[0].cpu().numpy(), o["x"]) < 1e-12


def test_cg_device_api_unaligned_vectors(nb):
    """Vectors one element off 16-byte alignment take the update's and
    glsc3's 8-byte (FP64) / 4-byte (FP32) paths: the same iterates as the
    aligned vectors' 16-byte paths, to rounding."""
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(3, 4, 3, 8, mask_mode=1)
    ctx = O.Ctx(3, 4, 3, 8, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n + 1, dtype=torch.float64, device=dev)
    f = torch.empty(n + 1, dtype=torch.float64, device=dev)
    m.setup_g(g.data_ptr())
    m.set_multiplicity(c[1:].data_ptr())
    m.rhs_uniform(f[1:].data_ptr(), c[1:].data_ptr(), 77)
    xs = []
    for off in (0, 1):
        fo = f[1:].clone() if off == 0 else f[1:]
        co = c[1:].clone() if off == 0 else c[1:]
        vs = [torch.zeros(n + 1, dtype=torch.float64, device=dev)[off:off + n] for _ in range(5)]
        assert (vs[0].data_ptr() % 16 == 0) == (off == 0)
        m.cg(*(t.data_ptr() for t in (vs[0], fo, g, co, vs[1], vs[2], vs[3], vs[4])), 60)
        xs.append(vs[0].cpu().numpy())
    o = ctx.cg(f[1:].cpu().numpy(), g.cpu().numpy(), c[1:].cpu().numpy(), 60)
    for x in xs:
        assert rel(x, o["x"]) < 1e-12
    assert rel(xs[0], xs[1]) < 1e-13
    # FP32 CG on unaligned vectors follows the aligned one to FP32 rounding
    f32, g32, c32 = f[1:].float(), g.float(), c[1:].float()
    hs = []
    for off in (0, 1):
        fo = f32.clone() if off == 0 else torch.zeros(n + 1, dtype=torch.float32, device=dev)
        if off == 1:
            fo[1:] = f32
            fo = fo[1:]
        co = c32.clone() if off == 0 else torch.zeros(n + 1, dtype=torch.float32, device=dev)
        if off == 1:
            co[1:] = c32
            co = co[1:]
        v = [torch.zeros(n + 1, dtype=torch.float32, device=dev)[off:off + n] for _ in range(4)]
        hs.append(m.cg_f32(v[0].data_ptr(), fo.data_ptr(), g32.data_ptr(), co.data_ptr(),
                           v[1].data_ptr(), v[2].data_ptr(), v[3].data_ptr(), 20, hist=True))
    assert np.allclose(hs[0][:, 0], hs[1][:, 0], rtol=1e-4)


def test_fp32_and_mixed_precision(nb):
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(4, 4, 4, 8, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    m.setup_g(g.data_ptr())
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 7)
    x64 = torch.zeros(n, dtype=torch.float64, device=dev)
    it, rr = m.cg_tol(x64.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10)
    assert rr <= 1e-10 and it > 10
    xm = torch.zeros(n, dtype=torch.float64, device=dev)
    outer, inner, rrm = m.cg_mixed(xm.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10, 20)
    assert rrm <= 1e-10 and outer >= 2
    assert (xm - x64).abs().max().item() <= 1e-8 * x64.abs().max().item()
    # fp32 CG alone follows the fp64 residual history while above fp32 noise
    f32, g32, c32 = f.float(), g.float(), c.float()
    v32 = [torch.zeros(n, dtype=torch.float32, device=dev) for _ in range(4)]
    h32 = m.cg_f32(v32[0].data_ptr(), f32.data_ptr(), g32.data_ptr(), c32.data_ptr(),
                   v32[1].data_ptr(), v32[2].data_ptr(), v32[3].data_ptr(), 30, hist=True)
    v64 = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(5)]
    h64 = m.cg(v64[0].data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), v64[1].data_ptr(),
               v64[2].data_ptr(), v64[3].data_ptr(), v64[4].data_ptr(), 30, hist=True)
    assert np.allclose(h32[:, 0], h64[:, 0], rtol=1e-3)


@pytest.mark.parametrize("deformed", [False, True])
def test_mixed_shared_metric_bitwise(nb, deformed):
    """The mixed solver's shared FP32 metric block (all elements equal, as
    setup_g makes them) gives bitwise the solution of per-element reads."""
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(6, 5, 4, 10, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    if deformed:
        m.setup_g_deformed(g.data_ptr(), 3, 0.1)
    else:
        m.setup_g(g.data_ptr())
        blk = g.view(-1, 6 * 10 ** 3)
        assert bool((blk == blk[0]).all())     # the box's blocks repeat
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 11)
    xs = {}
    try:
        for shared in (True, False):
            nb.set_shared_metric(shared)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            outer, inner, rr = m.cg_mixed(x.data_ptr(), f.data_ptr(), g.data_ptr(),
                                          c.data_ptr(), 1e-10, 20)
            assert rr <= 1e-10
            xs[shared] = (x.cpu().numpy(), outer)
    finally:
        nb.set_shared_metric(True)
    assert xs[True][1] == xs[False][1]
    assert np.array_equal(xs[True][0], xs[False][0])


@pytest.mark.parametrize("lx,inner,mask", [(10, 20, 1), (10, 7, 1), (7, 20, 1), (8, 20, 0)])
def test_mixed_inner_forms_bitwise(nb, lx, inner, mask):
    """The inner FP32 CG's streamlined forms give bitwise the solution and
    cycle count of the plain one: two direction buffers with one x update
    per pair of iterations (an odd inner count leaves its last iteration
    unpaired; odd lx1 takes the general operator), and c formed in closed
    form after it verified as the box's inverse multiplicity (even lx1; in
    either mask mode, since c does not depend on the mask).  Mask mode 0
    (the reference's element-1 quirk leaves most of the boundary free) is
    compared over six outer cycles, without a tolerance to reach."""
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(5, 4, 3, lx, mask_mode=mask)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    m.setup_g_deformed(g.data_ptr(), 5, 0.1)
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 13)
    # mask mode 0 masks every domain face on the mesh's first masking and
    # element 1's list after it (maskit's first-call branch): one solve
    # first, so that every compared solve sees the same mask
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    m.cg_mixed(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10, inner, 1)
    xs = {}
    try:
        for paired, closed in ((True, True), (False, True), (True, False), (False, False)):
            nb.set_paired_update(paired)
            nb.set_mixed_closed_multiplicity(closed)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            outer, tot, rr = m.cg_mixed(x.data_ptr(), f.data_ptr(), g.data_ptr(),
                                        c.data_ptr(), 1e-10, inner, 500 if mask else 6)
            assert rr <= 1e-10 or not mask
            xs[paired, closed] = (x.cpu().numpy(), outer, rr)
    finally:
        nb.set_paired_update(True)
        nb.set_mixed_closed_multiplicity(True)
    ref = xs[False, False]
    for key, got in xs.items():
        assert got[1:] == ref[1:], key
        assert np.array_equal(got[0], ref[0]), key


@pytest.mark.parametrize("niter", [9, 10])
@pytest.mark.parametrize("order", [2, 1])
def test_cg_paired_update_bitwise(nb, niter, order):
    """The FP64 CG with two direction buffers and one x update per pair of
    iterations gives bitwise the x, r, w, p, z and residual history of one
    buffer and an update every iteration, with the fixed-point (order 2) and
    the even-odd FP64 (order 1) operator; an even count ends with the last
    direction in the second buffer, copied to p."""
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(4, 3, 5, 8, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    m.setup_g_deformed(g.data_ptr(), 7, 0.1)
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 19)
    outs = {}
    try:
        m.set_order(order)
        for paired in (True, False):
            nb.set_paired_update(paired)
            x, r, w, p, z = (torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
                             for _ in range(5))
            h = m.cg(*(t.data_ptr() for t in (x, f, g, c, r, w, p, z)), niter, hist=True)
            torch.cuda.synchronize()
            outs[paired] = ([t.cpu().numpy() for t in (x, r, w, p, z)], h)
    finally:
        nb.set_paired_update(True)
        m.set_order(nb.DEFAULT_ORDER)
    for name, a, b in zip("xrwpz", outs[True][0], outs[False][0]):
        assert np.array_equal(a, b), name
    assert np.array_equal(outs[True][1], outs[False][1])


def test_kernel_timing_entry_points(nb):
    """nb_time_cg_kernels and nb_time_cg_kernels_f32 run the solvers' forms
    (paired x update on and off; FP32 with c formed in closed form) and
    report a positive time for each of the iteration's three kernels."""
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(4, 4, 4, 8, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    m.setup_g(g.data_ptr())
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 3)
    g32, c32, f32 = g.float(), c.float(), f.float()
    try:
        for paired in (True, False):
            nb.set_paired_update(paired)
            v = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(4)]
            ms = m.time_cg_kernels(v[0].data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(),
                                   v[1].data_ptr(), v[2].data_ptr(), v[3].data_ptr(), reps=2)
            v32 = [torch.zeros(n, dtype=torch.float32, device=dev) for _ in range(4)]
            ms32 = m.time_cg_kernels_f32(v32[0].data_ptr(), f32.data_ptr(), g32.data_ptr(),
                                         c32.data_ptr(), v32[1].data_ptr(), v32[2].data_ptr(),
                                         v32[3].data_ptr(), reps=2)
            assert len(ms) == 3 and all(t > 0 for t in ms), (paired, ms)
            assert len(ms32) == 3 and all(t > 0 for t in ms32), (paired, ms32)
            assert torch.isfinite(v[0]).all() and torch.isfinite(v32[0]).all()
    finally:
        nb.set_paired_update(True)


def test_mixed_closed_multiplicity_rejects_other_c(nb):
    """A c that is not the box's inverse multiplicity (one point changed)
    fails the closed-form check, and the inner CG reads it: the solve
    equals the one with the closed form switched off."""
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(4, 3, 3, 8, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    m.setup_g(g.data_ptr())
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 17)
    c[8 ** 3 * 5 + 4 + 8 * 3 + 64 * 2] = 0.75   # point (4,3,2) of element 5: interior
    xs = []
    try:
        for closed in (True, False):
            nb.set_mixed_closed_multiplicity(closed)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            outer, tot, rr = m.cg_mixed(x.data_ptr(), f.data_ptr(), g.data_ptr(),
                                        c.data_ptr(), 1e-9, 20, 60)
            xs.append((x.cpu().numpy(), outer, rr))
    finally:
        nb.set_mixed_closed_multiplicity(True)
    assert xs[0][1:] == xs[1][1:]
    assert np.array_equal(xs[0][0], xs[1][0])


# -------------------------------------------------------------------- hsmg --
@pytest.mark.parametrize("nx", [4, 5, 8, 10])
def test_h1mg_solve_matches_oracle(nb, nx):
    mesh = nb.Nekbone(3, 2, 2, nx, mask_mode=1)
    ctx = O.Ctx(3, 2, 2, nx, mask_mode=1)
    mesh.h1mg_setup()
    assert ctx.h1mg_setup() == 0
    rng = np.random.default_rng(8)
    rhs = rng.standard_normal(mesh.n)
    mesh.dssum(rhs)
    r1, r2 = rhs.copy(), rhs.copy()
    z = mesh.h1mg_solve(r1)
    zo = ctx.h1mg_solve(r2)
    assert rel(z, zo) < 1e-12
    # h1mg_solve masks its rhs in place, as the reference does
    assert np.array_equal(r1, r2)


def test_pcg_mgrid_matches_oracle(nb):
    mesh = nb.Nekbone(3, 3, 3, 8, mask_mode=1)
    ctx = O.Ctx(3, 3, 3, 8, mask_mode=1)
    c = mesh.set_multiplicity()
    g = mesh.setup_g()
    f = mesh.set_f(c)
    mesh.h1mg_setup()
    mesh.set_mgrid(True)
    ctx.h1mg_setup()
    x, r, w, p, z, _ = mesh.cg(f, g, c, 30)
    o = ctx.cg(f, g, c, 30, use_mg=True)
    mesh.set_mgrid(False)
    assert rel(x, o["x"]) < 1e-12

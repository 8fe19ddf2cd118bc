"""Deformed geometry (the deformed-box workloads): the device metric against a
numpy restatement, the FP64 operator on it against the oracle, and the error
of the FP32 operator against the FP64 oracle for lx1 in {8, 12, 16}.

Tolerances: the metric is computed with device sin/ and a different
evaluation order from numpy, so it must agree to 1e-13 relative.  The FP64
operator with a given metric is bit-exact in the reference order.  The FP32
operator's relative error against the FP64 oracle (max-norm, relative to
max|w|) is bounded by 2e-5.
"""
from __future__ import annotations

import numpy as np
import pytest

import geometry_ref as GR
import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _mesh_and_g(nb, torch, nel, lx, seed=11, amp=0.1):
    m = nb.DeviceMesh(nel, nel, nel, lx, mask_mode=1)
    g = torch.empty(6 * m.n, dtype=torch.float64, device="cuda")
    m.setup_g_deformed(g.data_ptr(), seed, amp)
    torch.cuda.synchronize()
    return m, g


def test_deformed_metric_matches_numpy(torch):
    import nekbone_gb300 as nb
    for nel, lx in ((3, 6), (2, 9)):
        m, g = _mesh_and_g(nb, torch, nel, lx)
        z, w = O.zwgll(lx)
        ref = GR.deformed_g(nel, nel, nel, z, w, seed=11, amp=0.1)
        got = g.cpu().numpy()
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) <= 1e-13 * scale
        # genuinely deformed: off-diagonal factors present, diagonal varies
        assert np.max(np.abs(ref.reshape(-1, 6)[:, 1])) > 1e-3 * scale


def test_deformed_metric_is_spd_and_operator_symmetric(torch):
    import nekbone_gb300 as nb
    m, g = _mesh_and_g(nb, torch, 3, 7)
    G = g.cpu().numpy().reshape(-1, 6)
    M = np.stack([np.stack([G[:, 0], G[:, 1], G[:, 2]], -1),
                  np.stack([G[:, 1], G[:, 3], G[:, 4]], -1),
                  np.stack([G[:, 2], G[:, 4], G[:, 5]], -1)], -2)
    assert np.all(np.linalg.eigvalsh(M) > 0)
    ctx = O.Ctx(3, 3, 3, 7, mask_mode=1)
    c = ctx.set_multiplicity()
    glo = O.set_vert_box(7, ctx.nelt, 3, 3, 3, ctx.lglel)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(glo.max() + 1)[glo]
    v = rng.standard_normal(glo.max() + 1)[glo]
    ctx.maskit(u)   # the masked operator is symmetric on masked vectors
    ctx.maskit(v)
    gh = np.ascontiguousarray(g.cpu().numpy())
    au, av = ctx.ax(u, gh), ctx.ax(v, gh)
    L = O.load()
    import ctypes as C
    a = L.orc_glsc3(O._p(v), O._p(c), O._p(au), C.c_int(ctx.n))
    b = L.orc_glsc3(O._p(u), O._p(c), O._p(av), C.c_int(ctx.n))
    assert abs(a - b) <= 1e-12 * abs(a)
    assert L.orc_glsc3(O._p(u), O._p(c), O._p(au), C.c_int(ctx.n)) > 0


@pytest.mark.parametrize("lx", [8, 12, 16])
def test_fp32_operator_error_vs_fp64_oracle(torch, lx):
    import nekbone_gb300 as nb
    nel = 4
    m, g = _mesh_and_g(nb, torch, nel, lx, seed=5)
    ctx = O.Ctx(nel, nel, nel, lx, mask_mode=1)
    glo = O.set_vert_box(lx, ctx.nelt, nel, nel, nel, ctx.lglel)
    rng = np.random.default_rng(lx)
    u = rng.uniform(-1, 1, glo.max() + 1)[glo]
    gh = np.ascontiguousarray(g.cpu().numpy())
    w64 = ctx.ax(u, gh)
    # FP64 device operator, reference order: bit-exact
    w = torch.empty(m.n, dtype=torch.float64, device="cuda")
    ut = torch.from_numpy(u).cuda()
    m.set_order(0)
    m.ax(w.data_ptr(), ut.data_ptr(), g.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy(), w64)
    m.set_order(nb.DEFAULT_ORDER)
    # FP32 operator
    w32 = torch.empty(m.n, dtype=torch.float32, device="cuda")
    u32, g32 = ut.float(), g.float()
    m.ax_f32(w32.data_ptr(), u32.data_ptr(), g32.data_ptr())
    torch.cuda.synchronize()
    err = np.max(np.abs(w32.cpu().numpy().astype(np.float64) - w64)) / np.max(np.abs(w64))
    print(f"lx1={lx}: FP32 operator max rel error vs FP64 oracle {err:.3e}")
    assert err < 2e-5


@pytest.mark.parametrize("lx", [4, 8, 10, 12, 16])
def test_tensor_core_operator_error_vs_fp64_oracle(torch, lx):
    """tcgen05 FP16 hi+lo split contractions with FP32 accumulation: the
    operator agrees with the FP64 oracle to FP32 accuracy (2e-5 relative,
    the same bound as the CUDA-core FP32 operator)."""
    import nekbone_gb300 as nb
    nel = 4 if lx <= 12 else 3
    m, g = _mesh_and_g(nb, torch, nel, lx, seed=5)
    ctx = O.Ctx(nel, nel, nel, lx, mask_mode=1)
    glo = O.set_vert_box(lx, ctx.nelt, nel, nel, nel, ctx.lglel)
    rng = np.random.default_rng(100 + lx)
    u = rng.uniform(-1, 1, glo.max() + 1)[glo]
    gh = np.ascontiguousarray(g.cpu().numpy())
    w64 = ctx.ax(u, gh)
    ut = torch.from_numpy(u).cuda().float()
    g32 = g.float()
    wt = torch.full((m.n,), float("nan"), dtype=torch.float32, device="cuda")
    m.ax_tc(wt.data_ptr(), ut.data_ptr(), g32.data_ptr())
    w32 = torch.empty(m.n, dtype=torch.float32, device="cuda")
    m.ax_f32(w32.data_ptr(), ut.data_ptr(), g32.data_ptr())
    torch.cuda.synchronize()
    got = wt.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(got))
    scale = np.max(np.abs(w64))
    err_tc = np.max(np.abs(got - w64)) / scale
    err_f32 = np.max(np.abs(w32.cpu().numpy().astype(np.float64) - w64)) / scale
    print(f"lx1={lx}: tensor-core operator max rel error {err_tc:.3e} (CUDA-core FP32 {err_f32:.3e})")
    assert err_tc < 2e-5

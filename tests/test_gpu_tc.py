"""Tensor-core (tcgen05) building blocks: one 128x16x16 MMA on small-integer
operands (exact in F16, BF16 and the FP32 accumulator) must reproduce the
exact product entry for entry."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bf16", [False, True])
def test_tcgen05_selftest_exact(bf16):
    import nekbone_gb300 as nb
    assert nb.tc_selftest(bf16) == 0


@pytest.mark.parametrize("dims,deformed", [((4, 3, 5, 8), False), ((3, 4, 3, 12), True),
                                           ((2, 3, 2, 7), True)])
def test_mixed_solver_with_tensor_core_inner_operator(dims, deformed):
    """The mixed solver with the inner CG's element products on the tensor
    cores reaches the tolerance through its FP64 defect correction, and its
    solution agrees with the CUDA-core mixed solution and the FP64 CG one."""
    import numpy as np
    torch = pytest.importorskip("torch")
    import nekbone_gb300 as nb
    m = nb.DeviceMesh(*dims, mask_mode=1)
    dev = torch.device("cuda")
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    if deformed:
        m.setup_g_deformed(g.data_ptr(), 9, 0.1)
    else:
        m.setup_g(g.data_ptr())
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 23)
    xs = {}
    try:
        for tc in (True, False):
            nb.set_mixed_tensor_cores(tc)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            outer, inner, rr = m.cg_mixed(x.data_ptr(), f.data_ptr(), g.data_ptr(),
                                          c.data_ptr(), 1e-10, 20, 200)
            assert rr <= 1e-10, (tc, outer, rr)
            xs[tc] = x.cpu().numpy()
    finally:
        nb.set_mixed_tensor_cores(False)
    xt = torch.zeros(n, dtype=torch.float64, device=dev)
    it, rr = m.cg_tol(xt.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                      max_iter=5000, check_every=10)
    assert rr <= 1e-10
    ref = xt.cpu().numpy()
    scale = np.abs(ref).max()
    assert np.abs(xs[True] - ref).max() <= 1e-8 * scale
    assert np.abs(xs[True] - xs[False]).max() <= 1e-8 * scale
    m.close()

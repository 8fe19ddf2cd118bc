"""Error paths of the device API: every rejected call fails with a status
(NekboneError) before it touches device memory, and the library stays
usable afterwards."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nb():
    import nekbone_gb300 as m
    return m


def test_mesh_size_and_argument_limits(nb):
    with pytest.raises(nb.NekboneError):
        nb.DeviceMesh(128, 128, 128, 16, mask_mode=1)   # 8.6e9 points > 2^31-1
    with pytest.raises(nb.NekboneError):
        nb.DeviceMesh(0, 2, 2, 6, mask_mode=1)
    with pytest.raises(nb.NekboneError):
        nb.DeviceMesh(2, 2, 2, 6, mask_mode=2)
    m = nb.DeviceMesh(2, 2, 2, 6, mask_mode=1)       # still usable
    assert m.n == 8 * 216
    m.close()


def test_multigrid_argument_checks(nb):
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(3, 3, 3, 8, mask_mode=1)
    with pytest.raises(nb.NekboneError):
        m.mg_setup([2, 4, 6], precision=64)            # finest order must be lx1-1
    with pytest.raises(nb.NekboneError):
        m.mg_setup([2, 4, 7], precision=16)            # 64 or 32
    with pytest.raises(nb.NekboneError):
        m.mg_setup([7], precision=64)                  # at least two levels
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device="cuda")
    m.setup_g(g.data_ptr())
    m.mg_setup([2, 4, 7], precision=64)
    with pytest.raises(nb.NekboneError):
        m.mg_setup_coarse(g.data_ptr())                # coarsest level not order 1
    m.close()


def test_exact_coarse_size_limit(nb):
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(32, 32, 32, 3, mask_mode=1)     # 31^3 coarse vertices
    g = torch.empty(6 * m.n, dtype=torch.float64, device="cuda")
    m.setup_g(g.data_ptr())
    m.mg_setup([1, 2], precision=64)
    with pytest.raises(nb.NekboneError):
        m.mg_setup_coarse(g.data_ptr())
    m.close()


def test_pcg_needs_multigrid_and_batch_checks(nb):
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(2, 2, 2, 6, mask_mode=1)
    n = m.n
    v = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(4)]
    g = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    with pytest.raises(nb.NekboneError):
        m.pcg_tol(v[0].data_ptr(), v[1].data_ptr(), g.data_ptr(), v[2].data_ptr(), 1e-10)
    m.close()
    b = nb.Batch([(2, 2, 2, 6), (1, 1, 2, 8)])
    with pytest.raises(nb.NekboneError):
        b.solve(1e-10, 20, 5)                          # before setup
    b.setup(3)
    with pytest.raises(nb.NekboneError):
        b.set_inner_tol(1.5)
    with pytest.raises(nb.NekboneError):
        b.solve(1e-10, 0, 5)
    b.solve(1e-10, 20, 20)                             # still usable
    nb.sync()
    assert all(b.result(p)[2] <= 1e-10 for p in range(b.nprob))
    b.close()


def test_bounded_wait_times_out_and_context_stays_usable(nb):
    """A device wait that nothing completes gives up after its poll limit:
    the call reports the timeout through the device error word, and the
    next calls on the same context run normally."""
    with pytest.raises(nb.NekboneError) as ei:
        nb.wait_selftest(256)
    assert "timed out" in str(ei.value)
    assert nb.tc_selftest() == 0
    a = np.arange(1.0, 9.0)
    assert nb.glsc3(a, a, np.ones(8)) == float((a * a).sum())
    nb.sync()
    with pytest.raises(nb.NekboneError):
        nb.wait_selftest(0)


def test_batched_metric_copy_timeout_is_reported(nb):
    """The batched FP32 operator brings each element's metric block in by a
    bulk copy.  With the wait self-test on, that wait runs out in every
    element: the solve's results are flagged (NB_ERR_CUDA from
    nb_batch_result) instead of being returned as valid, and after the
    switch is off a rebuilt solve is correct again on the same context."""
    probs = [(2, 2, 2, 6), (1, 1, 2, 8)]
    nb.set_wait_test(True)
    try:
        b = nb.Batch(probs)
        b.setup(5)
        b.solve(1e-10, 20, 5)
        with pytest.raises(nb.NekboneError) as ei:
            b.result(0)
        assert "timed out" in str(ei.value)
    finally:
        nb.set_wait_test(False)
    b.solve(1e-10, 20, 20)
    assert all(b.result(p)[2] <= 1e-10 for p in range(b.nprob))
    b.close()


def test_operator_metric_copy_timeout_is_reported(nb):
    """The same for the single-mesh FP32 operator with a per-element (here
    deformed) metric: nb_ax_f32 is asynchronous, so nb_sync reports the
    timeout; with the switch off the same call matches the FP64 operator."""
    torch = pytest.importorskip("torch")
    m = nb.DeviceMesh(2, 2, 2, 8, mask_mode=1)
    n = m.n
    g = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    m.setup_g_deformed(g.data_ptr(), 3, 0.1)
    u = torch.rand(n, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    g32, u32 = g.float(), u.float()
    w32 = torch.zeros(n, dtype=torch.float32, device="cuda")
    nb.set_wait_test(True)
    try:
        m.ax_f32(w32.data_ptr(), u32.data_ptr(), g32.data_ptr())
        with pytest.raises(nb.NekboneError) as ei:
            nb.sync()
        assert "timed out" in str(ei.value)
    finally:
        nb.set_wait_test(False)
    m.ax_f32(w32.data_ptr(), u32.data_ptr(), g32.data_ptr())
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    m.ax(w.data_ptr(), u.data_ptr(), g.data_ptr())
    nb.sync()
    err = float((w32.double() - w).abs().max() / w.abs().max())
    assert err < 1e-5
    m.close()

"""The gather-scatter topology of a box built on the device (closed-form
copies, no sort) against jl's sort-based construction on the host: the
gather-scatter CSR, the fused boundary groups with their mask flags and the
mask list must be identical, element for element; a CG solve on both meshes
must give bit-identical iterates."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOXES = [(3, 2, 2, 5), (4, 3, 2, 8), (2, 2, 2, 2), (1, 1, 1, 4), (5, 1, 1, 3), (1, 4, 1, 6),
         (3, 3, 3, 12)]


@pytest.fixture(scope="module")
def nb():
    import nekbone_gb300 as m
    yield m
    m.set_setup_on_device(True)


def _mesh(nb, dims, device):
    nb.set_setup_on_device(device)
    try:
        return nb.DeviceMesh(*dims, mask_mode=1)
    finally:
        nb.set_setup_on_device(True)


@pytest.mark.parametrize("dims", BOXES, ids=[f"{a}x{b}x{c}_lx{d}" for a, b, c, d in BOXES])
def test_device_topology_equals_host(nb, dims):
    md, mh = _mesh(nb, dims, True), _mesh(nb, dims, False)
    for getter in ("gs_maps", "boundary_groups"):
        od, idd = getattr(md, getter)()
        oh, idh = getattr(mh, getter)()
        assert np.array_equal(od, oh), getter
        assert np.array_equal(idd, idh), getter
    assert np.array_equal(md.mask_list(), mh.mask_list())
    md.close()
    mh.close()


def test_cg_identical_on_both_topologies(nb):
    torch = pytest.importorskip("torch")
    out = []
    for device in (True, False):
        m = _mesh(nb, (4, 3, 3, 7), device)
        n = m.n
        g = torch.empty(6 * n, dtype=torch.float64, device="cuda")
        c = torch.empty(n, dtype=torch.float64, device="cuda")
        f = torch.empty(n, dtype=torch.float64, device="cuda")
        m.setup_g(g.data_ptr())
        m.set_multiplicity(c.data_ptr())
        m.rhs_uniform(f.data_ptr(), c.data_ptr(), 3)
        x, r, w, p, z = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(5))
        m.cg(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), r.data_ptr(),
             w.data_ptr(), p.data_ptr(), z.data_ptr(), 30)
        torch.cuda.synchronize()
        out.append((c.cpu().numpy(), f.cpu().numpy(), x.cpu().numpy()))
        m.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_multigrid_on_device_topology(nb):
    """hsmg builds its host maps on demand when the mesh came from the device."""
    torch = pytest.importorskip("torch")
    res = []
    for device in (True, False):
        m = _mesh(nb, (3, 2, 2, 8), device)
        n = m.n
        g = torch.empty(6 * n, dtype=torch.float64, device="cuda")
        c = torch.empty(n, dtype=torch.float64, device="cuda")
        f = torch.empty(n, dtype=torch.float64, device="cuda")
        m.setup_g(g.data_ptr())
        m.set_multiplicity(c.data_ptr())
        m.rhs_uniform(f.data_ptr(), c.data_ptr(), 3)
        m.mg_setup([2, 4, 7], precision=64)
        z = torch.zeros_like(f)
        m.mg_solve(z.data_ptr(), f.clone().data_ptr())
        torch.cuda.synchronize()
        res.append(z.cpu().numpy())
        m.close()
    assert np.array_equal(res[0], res[1])

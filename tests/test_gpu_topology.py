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


def _mesh(nb, dims, device, mask_mode=1):
    nb.set_setup_on_device(device)
    try:
        return nb.DeviceMesh(*dims, mask_mode=mask_mode)
    finally:
        nb.set_setup_on_device(True)


def _box_numbering(nelx, nely, nelz, lx):
    """set_vert_box (prox_dssum.f:42-73) for the brick element order."""
    nn = lx - 1
    ax, ay = nn * nelx + 1, nn * nely + 1
    i = np.arange(lx)
    ez, ey, ex = np.meshgrid(np.arange(nelz), np.arange(nely), np.arange(nelx), indexing="ij")
    ig = (nn * ex.reshape(-1, 1, 1, 1) + i.reshape(1, 1, 1, lx))
    jg = (nn * ey.reshape(-1, 1, 1, 1) + i.reshape(1, 1, lx, 1))
    kg = (nn * ez.reshape(-1, 1, 1, 1) + i.reshape(1, lx, 1, 1))
    return (1 + ig + jg * ax + kg * ax * ay).astype(np.int64).ravel()


@pytest.mark.parametrize("mask_mode", [1, 0])
@pytest.mark.parametrize("dims", BOXES, ids=[f"{a}x{b}x{c}_lx{d}" for a, b, c, d in BOXES])
def test_device_topology_equals_host(nb, dims, mask_mode):
    md, mh = _mesh(nb, dims, True, mask_mode), _mesh(nb, dims, False, mask_mode)
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
    """hsmg set-up on a device-built mesh (its dssum on the device maps, no
    host maps at all) gives the host-built mesh's V-cycle, bit for bit."""
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


@pytest.mark.parametrize("dims", [(3, 2, 2, 5), (4, 3, 2, 8), (2, 2, 2, 2), (6, 1, 1, 2),
                                  (1, 4, 1, 6), (1, 1, 1, 4)])
def test_gs_setup_recognises_box_numbering(nb, dims):
    """gs_setup_ on set_vert_box's numbering builds its maps on the device;
    every gs_op result equals the host (jl sort-based) construction's, bit
    for bit.  A numbering one id away from a box goes the host way."""
    glo = _box_numbering(*dims)
    near = glo.copy()
    near[-1] = glo.max() + 7                       # no longer a box numbering
    rng = np.random.default_rng(2)
    for ids in (glo, near):
        res = {}
        for device in (True, False):
            nb.set_setup_on_device(device)
            try:
                h = nb.gs_setup(ids)
            finally:
                nb.set_setup_on_device(True)
            out = []
            for dtype in (np.float64, np.float32, np.int32, np.int64):
                for op in (1, 2, 3, 4):
                    for tr in (0, 1):
                        r = np.random.default_rng(op * 10 + tr)
                        u = (r.standard_normal(len(ids)) * 3).astype(dtype)
                        nb.gs_op(h, u, op, tr)
                        out.append(u)
            nb.gs_free(h)
            res[device] = out
        for a, b in zip(res[True], res[False]):
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_dropin_cg_on_recognised_box(nb):
    """The drop-in cg_ builds its operator on the device when gs_setup_ saw a
    box numbering; both mask modes give the host-built operator's iterates."""
    res = {}
    for device in (True, False):
        nb.set_setup_on_device(device)
        try:
            for mode in (0, 1):
                mesh = nb.Nekbone(3, 2, 2, 6, mask_mode=mode)
                g = mesh.setup_g()
                c = mesh.set_multiplicity()
                f = mesh.set_f(c)
                out = []
                for _ in range(2):                 # warm-up and timed call, driver.f:54-59
                    x = mesh.cg(f, g, c, 25)[0]
                    out.append(x.copy())
                res[(device, mode)] = out
        finally:
            nb.set_setup_on_device(True)
    for mode in (0, 1):
        for a, b in zip(res[(True, mode)], res[(False, mode)]):
            assert np.array_equal(a, b)

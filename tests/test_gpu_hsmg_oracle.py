"""hsmg as the C5 workload configures it, against the oracle.

C5 is hsmg-preconditioned CG at lx1 = 12 on deformed elements with the
levels 12 -> 6 -> 3 points ([2, 5, 11] in polynomial order), an FP64 or FP32
Schwarz smoother, and optionally the exact coarse solve.  Here:

* one V-cycle (h1mg_solve, hsmg.f:960-1034) with the FP64 smoother equals
  the oracle's restatement to 1e-12 (the two evaluate the same sums; they
  differ in summation order and in the eigensolvers behind the FDM, whose
  results agree to ~1e-15); with the FP32 smoother, to 1e-5 (FP32 rounding
  through ~10 tensor applies);
* preconditioned CG iterates with the FP64 smoother equal the oracle's PCG
  (cg.f:2-84 with h1mg_solve as solveM) to 1e-12; with the FP32 smoother,
  the solution to 1e-10 agrees with the oracle's FP64 PCG solution to 1e-8
  and its true residual, recomputed by the oracle's ax, is at the tolerance;
* the exact coarse solve is Galerkin: the difference it makes to a V-cycle
  equals P (Ac^-1 - I) P^T r, with P the trilinear interpolation from the
  interior vertices to the fine points and Ac = P^T A P built in numpy from
  the oracle's own ax.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu

C5_LEVELS = [2, 5, 11]


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.fixture(scope="module")
def nb():
    import nekbone_gb300 as m
    return m


def _threads():
    return max(1, min(16, os.cpu_count() or 1))


def _deformed(nb, torch, nel, lx, seed=7):
    m = nb.DeviceMesh(nel, nel, nel, lx, mask_mode=1)
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device="cuda")
    c = torch.empty(n, dtype=torch.float64, device="cuda")
    f = torch.empty(n, dtype=torch.float64, device="cuda")
    m.setup_g_deformed(g.data_ptr(), seed, 0.1)
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 99)
    torch.cuda.synchronize()
    return m, g, c, f


def _vcycle(m, torch, f):
    rhs = f.clone()
    z = torch.zeros_like(f)
    m.mg_solve(z.data_ptr(), rhs.data_ptr())
    torch.cuda.synchronize()
    return z.cpu().numpy()


@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 1e-5)])
def test_c5_vcycle_matches_oracle(nb, torch, precision, tol):
    m, g, c, f = _deformed(nb, torch, 3, 12)
    m.mg_setup(C5_LEVELS, precision=precision)
    ctx = O.Ctx(3, 3, 3, 12, mask_mode=1, nthreads=_threads())
    assert ctx.h1mg_setup(C5_LEVELS) == 0
    assert ctx.h1mg_levels() == C5_LEVELS
    z = _vcycle(m, torch, f)
    zo = ctx.h1mg_solve(f.cpu().numpy().copy())
    err = np.max(np.abs(z - zo)) / np.max(np.abs(zo))
    print(f"C5 V-cycle, FP{precision} smoother: {err:.3e}")
    assert err <= tol
    m.close()


def test_c5_pcg_fp64_smoother_matches_oracle(nb, torch):
    m, g, c, f = _deformed(nb, torch, 3, 12)
    m.mg_setup(C5_LEVELS, precision=64)
    ctx = O.Ctx(3, 3, 3, 12, mask_mode=1, nthreads=_threads())
    ctx.h1mg_setup(C5_LEVELS)
    niter = 30
    vs = [torch.zeros_like(f) for _ in range(5)]
    hist = m.cg(*(t.data_ptr() for t in (vs[0], f, g, c, vs[1], vs[2], vs[3], vs[4])), niter,
                flags=2, hist=True)
    o = ctx.cg(f.cpu().numpy(), g.cpu().numpy(), c.cpu().numpy(), niter, use_mg=True)
    x = vs[0].cpu().numpy()
    err = np.max(np.abs(x - o["x"])) / np.max(np.abs(o["x"]))
    print(f"C5 PCG x after {niter}: {err:.3e}")
    assert err <= 1e-12
    assert np.allclose(hist[:, 0], o["hist"][:, 0], rtol=1e-10, atol=0)
    m.close()


def test_c5_pcg_fp32_smoother_solution_and_residual(nb, torch):
    m, g, c, f = _deformed(nb, torch, 3, 12)
    ctx = O.Ctx(3, 3, 3, 12, mask_mode=1, nthreads=_threads())
    ctx.h1mg_setup(C5_LEVELS)
    o = ctx.cg(f.cpu().numpy(), g.cpu().numpy(), c.cpu().numpy(), 200, use_mg=True)
    m.mg_setup(C5_LEVELS, precision=32)
    x = torch.zeros_like(f)
    it, rr = m.pcg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                       max_iter=500, check_every=1)
    assert rr <= 1e-10
    xh, fh, ch = x.cpu().numpy(), f.cpu().numpy(), c.cpu().numpy()
    assert np.max(np.abs(xh - o["x"])) <= 1e-8 * np.max(np.abs(o["x"]))
    res = fh - ctx.ax(xh, g.cpu().numpy())
    ctx.maskit(res)
    true_rel = np.sqrt(np.sum(res * ch * res)) / np.sqrt(np.sum(fh * ch * fh))
    print(f"C5 PCG FP32 smoother: {it} iterations, relres {rr:.3e}, oracle {true_rel:.3e}")
    assert true_rel <= 1.01e-10
    m.close()


def _interior_vertex_interpolation(nel, lx):
    """P: local fine points x interior vertices of a nel^3 brick, the
    trilinear hat function of each interior vertex at every element's GLL
    points (element ex fastest, points i fastest)."""
    z, _ = O.zwgll(lx)
    phi = np.stack([(1 - z) / 2, (1 + z) / 2])          # phi[a][i]
    nv = nel + 1
    inner = [(vx, vy, vz) for vz in range(1, nel) for vy in range(1, nel)
             for vx in range(1, nel)]
    col = {v: q for q, v in enumerate(inner)}
    l3 = lx ** 3
    P = np.zeros((nel ** 3 * l3, len(inner)))
    for ez in range(nel):
        for ey in range(nel):
            for ex in range(nel):
                e = ex + nel * (ey + nel * ez)
                for cz in range(2):
                    for cy in range(2):
                        for cx in range(2):
                            v = (ex + cx, ey + cy, ez + cz)
                            if v not in col:
                                continue
                            hat = np.einsum("k,j,i->kji", phi[cz], phi[cy], phi[cx]).reshape(-1)
                            P[e * l3:(e + 1) * l3, col[v]] += hat
    assert nv > 2
    return P


@pytest.mark.parametrize("levels", [[1, 3, 5], [1, 5]])
def test_exact_coarse_is_galerkin(nb, torch, levels):
    """With the FP64 smoother, a V-cycle with the exact coarse solve minus
    the same V-cycle with the reference's dssum coarse step (both additive,
    their smoother parts bitwise equal) is P (Ac^-1 - I) P^T r, where
    P^T r is the assembled restricted residual and the dssum step returns it
    unchanged."""
    nel, lx = 3, 6
    m, g, c, f = _deformed(nb, torch, nel, lx, seed=13)
    m.mg_setup(levels, precision=64)
    z_dssum = _vcycle(m, torch, f)
    m.mg_setup(levels, precision=64)
    m.mg_setup_coarse(g.data_ptr())
    z_exact = _vcycle(m, torch, f)
    # Ac = P^T A P from the oracle's ax (global inner products: the local
    # vectors are continuous, so each global point is weighted by 1/mult)
    ctx = O.Ctx(nel, nel, nel, lx, mask_mode=1)
    gh, ch, fh = g.cpu().numpy(), c.cpu().numpy(), f.cpu().numpy()
    P = _interior_vertex_interpolation(nel, lx)
    AP = np.stack([ctx.ax(P[:, j].copy(), gh) for j in range(P.shape[1])], axis=1)
    Ac = P.T @ (ch[:, None] * AP)
    assert np.allclose(Ac, Ac.T, rtol=1e-12, atol=1e-14 * np.abs(Ac).max())
    r = fh.copy()
    ctx.maskit(r)
    b = P.T @ (ch * r)
    dz = P @ (np.linalg.solve(Ac, b) - b)
    got = z_exact - z_dssum
    err = np.max(np.abs(got - dz)) / np.max(np.abs(dz))
    print(f"exact coarse, levels {levels}: {err:.3e}")
    assert np.max(np.abs(dz)) > 1e-3 * np.max(np.abs(z_exact))   # the coarse part matters
    assert err <= 1e-12
    m.close()

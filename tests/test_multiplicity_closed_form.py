"""The premise of the inner CGs' closed-form multiplicity (no GPU).

The mixed solver and the batched solve form the FP32 inverse multiplicity c
instead of reading it once a check pass has verified, bitwise at every point,
that c = 2^-m: m counts the point's extreme local indices (i, j or k equal to
0 or lx1-1) on element faces that have a neighbour, and a face has one where c
at its point (1, 1) is 1/2 (k_c_closed_form, k_bc_closed_form).  These tests
restate that rule in numpy and check it against the oracle's own
set_multiplicity on box meshes of both mask modes, and that it rejects
multiplicities of another form, so a verified c is the box's c.  They also
check the index tracking the update kernels use to find each 16-byte group's
element and position without a division per group.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O


def _ext_bits(lx: int) -> np.ndarray:
    """Extreme-index bits of an element's points (bit 0/1: i = 0 / lx-1,
    2/3 for j, 4/5 for k), in the kernels' point order i + lx j + lx^2 k."""
    l = np.arange(lx ** 3)
    i, j, k = l % lx, (l // lx) % lx, l // (lx * lx)
    return ((i == 0) * 1 | (i == lx - 1) * 2 | (j == 0) * 4 | (j == lx - 1) * 8 |
            (k == 0) * 16 | (k == lx - 1) * 32).astype(np.uint32)


def _face_bits(ce: np.ndarray, lx: int) -> np.ndarray:
    """Each element's face bits from c at the face points (1, 1)."""
    m, h, L2 = 1, lx - 1, lx * lx
    pts = [0 + lx * m + L2 * m, h + lx * m + L2 * m, m + L2 * m,
           m + lx * h + L2 * m, m + lx * m, m + lx * m + L2 * h]
    fb = np.zeros(ce.shape[0], dtype=np.uint32)
    for f, pt in enumerate(pts):
        fb |= np.where(ce[:, pt] == np.float32(0.5), np.uint32(1 << f), np.uint32(0))
    return fb


def _closed_form(c32: np.ndarray, lx: int, nelt: int) -> tuple[np.ndarray, bool]:
    ce = c32.reshape(nelt, lx ** 3)
    fb = _face_bits(ce, lx)
    both = fb[:, None] & _ext_bits(lx)[None, :]
    m = np.zeros(both.shape, dtype=np.int64)
    for bit in range(6):
        m += (both >> bit) & 1
    want = np.ldexp(np.float32(1.0), -m).astype(np.float32)
    return fb, bool(np.array_equal(want.view(np.uint32), ce.view(np.uint32)))


@pytest.mark.parametrize("dims", [(5, 4, 3, 10), (3, 3, 3, 8), (4, 4, 4, 12), (2, 1, 1, 4),
                                  (1, 1, 1, 6), (1, 3, 1, 16)])
@pytest.mark.parametrize("mask_mode", [0, 1])
def test_box_multiplicity_is_closed_form(dims, mask_mode):
    nx, ny, nz, lx = dims
    ctx = O.Ctx(nx, ny, nz, lx, mask_mode=mask_mode)
    c = ctx.set_multiplicity().astype(np.float32)
    fb, ok = _closed_form(c, lx, nx * ny * nz)
    assert ok
    # a face has a neighbour exactly when the element is not on that side of
    # the box (brick element order: x fastest)
    e = np.arange(nx * ny * nz)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    want = ((ex > 0) * 1 | (ex < nx - 1) * 2 | (ey > 0) * 4 | (ey < ny - 1) * 8 |
            (ez > 0) * 16 | (ez < nz - 1) * 32).astype(np.uint32)
    assert np.array_equal(fb, want)


def test_other_multiplicities_are_rejected():
    lx, nelt = 8, 3 * 2 * 2
    ctx = O.Ctx(3, 2, 2, lx, mask_mode=1)
    c = ctx.set_multiplicity().astype(np.float32)
    assert _closed_form(c, lx, nelt)[1]
    for q, v in ((5 * lx ** 3 + 4 + lx * 3 + lx * lx * 2, 0.75),   # interior point
                 (0, 0.5),                                           # a corner
                 (lx ** 3 - 1, np.float32(1.0 / 3.0))):
        bad = c.copy()
        bad[q] = v
        assert not _closed_form(bad, lx, nelt)[1], q
    assert not _closed_form(np.full_like(c, 0.5), lx, nelt)[1]


@pytest.mark.parametrize("lx", [4, 6, 8, 10, 12, 16])
def test_group_index_tracking(lx):
    """(element, group) of a thread's 16-byte groups, advanced by the
    stride's quotient and remainder as k_cg_update (grid-stride) and k_bupd
    (2048-point chunks of one problem) do, equals divmod(v, lx^3/4)."""
    q4 = lx ** 3 // 4
    for nelt, stride in ((7, 256), (40, 3 * 256), (130, 1216 * 256)):
        nv = nelt * q4
        for v0 in (0, 5, min(stride, nv) - 1):
            e, l4 = divmod(v0, q4)
            se, sl = divmod(stride, q4)
            v = v0
            while v < nv:
                assert (e, l4) == divmod(v, q4)
                l4 += sl
                e += se
                if l4 >= q4:
                    l4 -= q4
                    e += 1
                v += stride
    # chunks of 2048 points within a problem that starts at point pt0
    pt0, kthreads, chunk = 4 * 1000, 256, 2048
    n = 27 * lx ** 3
    for a in range(0, n, chunk):
        q0, q1 = pt0 + a, pt0 + min(a + chunk, n)
        for tid in (0, 1, 97, 255):
            vrel = (q0 - pt0) // 4 + tid
            le, l4 = divmod(vrel, q4)
            se, sl = divmod(kthreads, q4)
            v = q0 // 4 + tid
            while v < q1 // 4:
                assert (le, l4) == divmod(v - pt0 // 4, q4)
                l4 += sl
                le += se
                if l4 >= q4:
                    l4 -= q4
                    le += 1
                v += kthreads

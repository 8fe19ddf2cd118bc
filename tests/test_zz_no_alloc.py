"""The allocation-free glsc3 (nb_glsc3_noalloc) against the library's
ordinary glsc3_, through the C ABI.

nb_glsc3_noalloc exists for callers that may not call cudaMalloc while they
run (their device memory belongs to their own pool, or an allocation's
implicit device synchronisation is not allowed in their loop).  It keeps its
reduction scratch in a fixed device array of the library instead of
allocating.  This file is collected last so that a failure here comes after
every other test has run.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_glsc3_noalloc_matches_glsc3_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    import nekbone_gb300 as nb

    rng = np.random.default_rng(2027)
    # the second call is smaller than the first: nothing the first call left
    # in the shared scratch may leak into it
    for n in (3_000_017, 4099):
        a, b, m = rng.standard_normal(n), rng.standard_normal(n), rng.random(n)
        expect = nb.glsc3(a, b, m)
        ta, tb, tm = (torch.from_numpy(x).cuda() for x in (a, b, m))
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        status = nb.lib.nb_glsc3_noalloc(ta.data_ptr(), tb.data_ptr(), tm.data_ptr(), n,
                                         out.data_ptr(), None)
        assert status == 0, nb.lib.nekbone_last_message()
        torch.cuda.synchronize()
        got = out.item()
        # both are FP64 reductions that differ only in summation order
        assert abs(got - expect) <= 1e-12 * float(np.sum(np.abs(a * b * m)))


def test_glsc3_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    import nekbone_gb300 as nb

    t = torch.zeros(4, dtype=torch.float64, device="cuda")
    status = nb.lib.nb_glsc3_noalloc(t.data_ptr(), t.data_ptr(), t.data_ptr(),
                                     nb.NOALLOC_MAX_N + 1, t.data_ptr(), None)
    assert status == 1
    assert b"outside" in nb.lib.nekbone_last_message()
    nb.lib.nekbone_clear_status()


def test_glsc3_noalloc_empty_and_on_a_callers_stream():
    """n = 0 writes 0.0 (its own path: no kernel); and a call enqueued on a
    stream of the caller's, passed as its handle, gives glsc3_'s value once
    that stream is synchronised."""
    torch = pytest.importorskip("torch")
    import nekbone_gb300 as nb

    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert nb.lib.nb_glsc3_noalloc(None, None, None, 0, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert out.item() == 0.0

    rng = np.random.default_rng(31)
    n = 1_000_003
    a, b, m = rng.standard_normal(n), rng.standard_normal(n), rng.random(n)
    expect = nb.glsc3(a, b, m)
    ta, tb, tm = (torch.from_numpy(x).cuda() for x in (a, b, m))
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    out.fill_(float("nan"))
    torch.cuda.synchronize()
    status = nb.lib.nb_glsc3_noalloc(ta.data_ptr(), tb.data_ptr(), tm.data_ptr(), n,
                                     out.data_ptr(), side.cuda_stream)
    assert status == 0, nb.lib.nekbone_last_message()
    side.synchronize()
    assert abs(out.item() - expect) <= 1e-12 * float(np.sum(np.abs(a * b * m)))

"""Tensor-core (tcgen05) building blocks: one 128x16x16 MMA on small-integer
operands (exact in F16, BF16 and the FP32 accumulator) must reproduce the
exact product entry for entry."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bf16", [False, True])
def test_tcgen05_selftest_exact(bf16):
    import nekbone_gb300 as nb
    assert nb.tc_selftest(bf16) == 0

"""The exact rewrites of the FP64 decision path against CUDA's own operations: division by
a known reciprocal with one Markstein correction, float-to-double and integer-to-double by
integer operations, ordered comparisons of doubles by integer operations, and the
binary32-first Metropolis test.  Any mismatch would break bit-exactness."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2])
def test_exact_rewrites_match_cuda(gpu, seed):
    n = 1 << 30
    mism, first = gpu.check_numerics(n, seed)
    assert int(mism[0]) == 0, ("division", first)
    assert int(mism[1]) == 0, "float to double"
    assert int(mism[2]) == 0, "Metropolis"
    assert int(mism[3]) == 0, "ordered comparison by integer instructions"
    assert int(mism[4]) == 0, "integer to double by integer instructions"

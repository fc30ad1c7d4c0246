"""GPU: the integer-pipe FP64 multiply the sweeps use equals the FP64 unit
bit for bit (random significands, ties to even, zeros, subnormals,
infinities, NaN, extreme exponents)."""
import pytest

from ramgpu import abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_integer_multiply_matches_fp64_unit(seed):
    assert abi.selftest_arith(4_000_000, seed) == 0

"""The kernels' integer-pipe binary64 product and quotient (fp64ops.cuh: mulI, divI)
are bit-identical to the FP64 unit's, over seeded operands of every class; the
bit-pattern limiters (common.cuh) equal their expressions."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_integer_pipe_mul_div_match_fp64_unit(hg, seed):
    mul_bad, div_bad = hg.fp64_selftest(cases=1 << 27, seed=seed)
    assert (mul_bad, div_bad) == (0, 0)


@pytest.mark.parametrize("seed", [1, 2])
def test_bit_pattern_limiters_match_their_expressions(hg, seed):
    """MinMod and Superbee decided on the bit patterns give the fmin/fmax chains'
    results bit for bit (signs of zero included) on ratios of every class."""
    assert hg.limiter_selftest(cases=1 << 26, seed=seed) == 0

"""The kernels' integer-pipe binary64 product and quotient (fp64ops.cuh: mulI, divI)
are bit-identical to the FP64 unit's, over seeded operands of every class."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_integer_pipe_mul_div_match_fp64_unit(hg, seed):
    mul_bad, div_bad = hg.fp64_selftest(cases=1 << 27, seed=seed)
    assert (mul_bad, div_bad) == (0, 0)

"""The GPU's results against the FP64 oracle, per result type, through the
C-ABI (same cases and bounds as the FP32-oracle statement)."""
import pytest

from tests.test_oracle_precision import BOUND, fp64_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("three_d", [False, True])
def test_gpu_error_against_fp64_oracle(ctx, oracle, three_d):
    def run32(g, vel, sou, w, rec, m):
        return {"modeling": lambda: ctx.modeling(g, vel, sou, w, rec),
                "born": lambda: ctx.born(g, vel, m, sou, w, rec),
                "rtm": lambda d: ctx.rtm(g, vel, sou, w, rec, d),
                "lsrtm": lambda d: ctx.lsrtm(g, vel, sou, w, rec, d)[0]}
    err = fp64_errors(oracle, three_d, run32)
    for k, e in err.items():
        assert 0 < e < BOUND[k][int(three_d)], (k, e)

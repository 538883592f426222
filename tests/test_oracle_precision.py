"""Each result's error against the FP64 oracle, stated.

The FP32 restatement of the oracle evaluates every expression in the same
order as the CUDA kernels (the GPU parity tests assert bit-for-bit equality
between the two), so its distance to the FP64 twin of the same algorithm is
the GPU's error against FP64.  The test asserts a bound a few times the
measured figure; the measured figures are (relative L2, max-abs relative):

    result                 2D (60x80, nt 400)      3D (30x36x32, nt 120)
    modeling traces        9.9e-6 / 3.1e-6         3.8e-6 / 1.6e-6
    Born traces            2.7e-5 / 1.1e-5         4.5e-6 / 3.9e-6
    RTM image              7.4e-6 / 3.6e-6         3.4e-6 / 5.6e-7
    RTM illumination       2.1e-6 / 6.4e-7         2.3e-7 / 1.8e-7
    LSRTM image            6.7e-6 / 3.4e-6         3.3e-6 / 5.5e-7
"""
import numpy as np
import pytest

from tests.cases import case2d, case3d

BOUND = {   # (2D, 3D) relative L2 bounds
    "modeling": (5e-5, 2e-5),
    "born": (1e-4, 2.5e-5),
    "rtm_image": (4e-5, 2e-5),
    "rtm_illum": (1e-5, 2e-6),
    "lsrtm_image": (4e-5, 2e-5),
}


def _rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def fp64_errors(oracle, three_d, run32=None):
    """Relative L2 error of every result type against the FP64 oracle.
    `run32` computes the FP32 results (default: the FP32 oracle)."""
    g, vel, sou, rec, w = case3d(nt=120) if three_d else case2d(nt=400)
    rng = np.random.default_rng(5)
    m = rng.standard_normal(vel.shape).astype(np.float32)
    if run32 is None:
        run32 = {"modeling": lambda: oracle.modeling(g, vel, sou, w, rec),
                 "born": lambda: oracle.born(g, vel, m, sou, w, rec),
                 "rtm": lambda d: oracle.rtm(g, vel, sou, w, rec, d),
                 "lsrtm": lambda d: oracle.lsrtm(g, vel, sou, w, rec, d)[0]}
    else:
        run32 = run32(g, vel, sou, w, rec, m)
    d32 = run32["modeling"]()
    d64 = oracle.modeling(g, vel, sou, w, rec, f64=True)
    b64 = oracle.born(g, vel, m, sou, w, rec, f64=True)
    # The imaging inputs are the FP32 traces so that the two runs migrate
    # the same data.
    r32, i32 = run32["rtm"](d32)
    r64, i64 = oracle.rtm(g, vel, sou, w, rec, d32, f64=True)
    l32 = run32["lsrtm"](d32)
    l64, _ = oracle.lsrtm(g, vel, sou, w, rec, d32, f64=True)
    return {"modeling": _rel(d32, d64), "born": _rel(run32["born"](), b64),
            "rtm_image": _rel(r32, r64), "rtm_illum": _rel(i32, i64),
            "lsrtm_image": _rel(l32, l64)}


@pytest.mark.parametrize("three_d", [False, True])
def test_fp32_error_against_fp64_oracle(oracle, three_d):
    err = fp64_errors(oracle, three_d)
    for k, e in err.items():
        assert 0 < e < BOUND[k][int(three_d)], (k, e)

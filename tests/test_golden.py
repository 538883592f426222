"""The committed golden fixtures (tests/golden/*.npz, written by
tests/golden/make_golden.py from the FP32 oracle) against the oracle on the
CPU and against the device path through the C-ABI."""
import glob
import os

import numpy as np
import pytest

from tests.conftest import rel_l2
from tests.golden.golden_cases import run

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
NAMES = [os.path.splitext(os.path.basename(p))[0] for p in GOLDEN]


def _load(path):
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def test_fixture_set_is_complete():
    assert set(NAMES) >= {"modeling2d", "modeling3d", "rtm2d", "rtm3d", "born2d", "lsrtm2d",
                          "fwi2d", "rho_modeling2d", "rho_afwi2d", "rho_modeling3d",
                          "surface_modeling2d", "afwi2d", "born3d", "lsrtm3d"}


@pytest.mark.parametrize("path", GOLDEN, ids=NAMES)
def test_oracle_reproduces_golden(oracle, path):
    fx = _load(path)
    out = run(oracle, fx)
    assert out.keys() == {k for k in fx if k.startswith("out_")}
    for k, v in out.items():
        assert np.abs(fx[k]).max() > 0, k
        np.testing.assert_array_equal(v, fx[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=NAMES)
def test_device_reproduces_golden(ctx, path):
    """Bit-exact for traces, wavefields and images; the FWI gradient and
    illumination pass through one FP64 norm summed in a different order on
    the device, so they are held to 1e-6 relative L2 (the misfit is exact)."""
    fx = _load(path)
    out = run(ctx, fx)
    for k, v in out.items():
        if str(fx["kind"]) == "fwi" and k in ("out_gradient", "out_illum"):
            assert rel_l2(v, fx[k]) < 1e-6, k
        else:
            np.testing.assert_array_equal(v, fx[k], err_msg=k)

"""FWI data preprocessing on the GPU: the band-pass of sw_bandpass against the
oracle's restatement, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flo,fhi,phase", [(0.0, 20.0, 0), (6.0, 25.0, 0), (6.0, 25.0, 1),
                                           (3.0, 240.0, 0)])
def test_bandpass_matches_oracle(ctx, oracle, flo, fhi, phase):
    rng = np.random.default_rng(4)
    tr = rng.standard_normal((257, 700)).astype(np.float32)
    a = ctx.bandpass(tr, 2e-3, flo=flo, fhi=fhi, phase=phase)
    b = oracle.bandpass(tr, 2e-3, flo=flo, fhi=fhi, phase=phase)
    assert np.abs(b).max() > 0
    np.testing.assert_array_equal(a, b)

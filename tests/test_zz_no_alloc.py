"""sw_modeling_noalloc against sw_modeling (GPU, through the C ABI).

Collected last on purpose: it must pass in a fresh process and after every
other GPU test (whose buffers may still occupy the device).  The two calls
in a row use different shots, so the second call also shows that the shared
scratch array is cleared between calls.
"""
import numpy as np
import pytest

import seismic_gb300 as sw
from tests.cases import case2d


@pytest.mark.gpu
def test_modeling_noalloc_matches_modeling_twice(ctx):
    g, vel, sou, rec, w = case2d(nz=60, nx=80, nt=300, seed=3)
    sou2 = sou.copy()
    sou2[1] = 13 * 10.0 + 4.2
    for s in (sou, sou2):
        ref = ctx.modeling(g, vel, s, w, rec)
        out = sw.modeling_noalloc(g, vel, s, w, rec)
        assert np.abs(ref).max() > 0
        # Same kernels and operation order as every modelling parity test:
        # bit-exact.
        np.testing.assert_array_equal(out, ref)


@pytest.mark.gpu
def test_modeling_noalloc_rejects_oversize(ctx):
    # 2000 x 2000 padded grid: six float arrays need ~100 MB > 32 MiB.
    g, vel, sou, rec, w = case2d(nz=60, nx=80, nt=8, seed=0)
    big = sw.make_genpar(1960, 1960, 1, dz=10.0, dx=10.0, dt=1.5e-3, nt=8, ntaper=10, lsinc=7,
                         snapi=4, fmax=30.0)
    vbig = np.full((1960, 1960), 2000.0, np.float32)
    with pytest.raises(sw.SwaveError) as ei:
        sw.modeling_noalloc(big, vbig, sou, w, rec)
    assert ei.value.code == sw.SW_OOM_ADMISSION


@pytest.mark.gpu
@pytest.mark.parametrize("field", ["surf_type", "shot_type", "rec_type"])
def test_modeling_noalloc_rejects_surface_and_mirror_modes(ctx, field):
    # The free surface and the mirror modes are built on the allocating
    # entry points only; this one refuses them instead of ignoring them.
    g, vel, sou, rec, w = case2d(nz=60, nx=80, nt=8, seed=0)
    setattr(g, field, 1)
    with pytest.raises(sw.SwaveError) as ei:
        sw.modeling_noalloc(g, vel, sou, w, rec)
    assert ei.value.code == sw.SW_UNSUPPORTED

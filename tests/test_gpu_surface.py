"""Free surface and mirror sources/receivers on the GPU against the oracle,
bit for bit: modelling (sinc and nearest-node extraction), the snapshots and
RTM images under a free surface, 2D and 3D."""
import numpy as np
import pytest

import seismic_gb300 as sw
from tests.cases import case2d, case3d

pytestmark = pytest.mark.gpu


def _types(g, surf, shot, rec, oz=None):
    g.surf_type, g.shot_type, g.rec_type = surf, shot, rec
    if oz is not None:
        g.oz = oz
    return g


@pytest.mark.parametrize("surf,shot,rec,oz,ext", [
    (1, 0, 0, 0.0, sw.EXT_SINC),          # free surface on a row
    (1, 0, 0, -4.0, sw.EXT_SINC),         # free surface between rows (sinc mirror)
    (0, 1, 1, 0.0, sw.EXT_SINC),          # mirror source and receivers
    (0, 1, 1, 0.0, sw.EXT_SIMPLE_AFWI),   # mirror nearest-node receivers
    (1, 1, 0, 0.0, sw.EXT_SINC),          # both
])
def test_modeling_with_surface_types(ctx, oracle, surf, shot, rec, oz, ext):
    g, vel, sou, rec_c, w = case2d(nt=300)
    g = _types(g, surf, shot, rec, oz)
    sou = np.array([20.4, sou[1], 0.0], np.float32)   # mirror footprint inside the grid
    rec_c[:, 0] = 20.7
    d = sw.SwPropDesc()
    d.g = g
    d.tmin, d.tmax, d.tstep = 1, g.nt, 1
    d.fd_scheme, d.injection, d.extraction = sw.FD_FORWARD, sw.INJ_SINC, ext
    a = np.zeros((rec_c.shape[0], g.nt), np.float32)
    b = np.zeros_like(a)
    ctx.propagate(d, vel, sou, w, rec_c, a)
    oracle.propagate(d, vel, sou, w, rec_c, b)
    assert np.abs(b).max() > 0
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("three_d", [False, True])
def test_rtm_under_a_free_surface(ctx, oracle, three_d):
    """Snapshots keep zeros above the surface row and the imaging starts at
    it (Extraction.f90:580-592, Imaging.f90:248-258); the backward pass
    injects through mirror receivers."""
    g, vel, sou, rec, w = case3d(nt=80) if three_d else case2d(nt=200)
    g = _types(g, 1, 0, 1, -12.0)
    sou = np.array([25.0, sou[1], sou[2]], np.float32)
    rec[:, 0] = 5.0      # shallow enough for the mirror to stay in the grid
    data = (np.random.default_rng(3).standard_normal((rec.shape[0], g.nt)) * 1e-2).astype(np.float32)
    n = vel.size
    out = {}
    for name, api in (("gpu", ctx), ("oracle", oracle)):
        wave = np.zeros((g.nt // g.snapi) * n, np.float32)
        f = sw.SwPropDesc()
        f.g = g
        f.tmin, f.tmax, f.tstep = 1, g.nt, 1
        f.fd_scheme, f.injection, f.extract_wave = sw.FD_FORWARD, sw.INJ_SINC, 1
        api.propagate(f, vel, sou, w, wave=wave)
        bk = sw.SwPropDesc()
        bk.g = g
        bk.tmin, bk.tmax, bk.tstep = g.nt, 1, -1
        bk.fd_scheme = sw.FD_FORWARD if three_d else sw.FD_ADJOINT
        bk.injection, bk.imaging = sw.INJ_SINC, sw.IMG_RTM
        im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
        api.propagate(bk, vel, rec, data, wave=wave, image=im, illum=il)
        out[name] = (wave, im, il)
    wave = out["oracle"][0].reshape(g.nt // g.snapi, *vel.shape)
    # the surface row is 2 (oz = -12 m): row 1 is stored as zero
    assert np.abs(wave[..., 0]).max() == 0 and np.abs(wave[..., 1]).max() > 0
    for q in range(3):
        np.testing.assert_array_equal(out["gpu"][q], out["oracle"][q])

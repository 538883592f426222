"""The variable-density path on the GPU (withRho: the staggered
FD_{2D,3D}_derivatives_acoustic_forward_grid operator, v^2*rho injection)
against the oracle, bit for bit, through sw_propagate and the SEP modelling
program."""
import subprocess

import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300 import sep
from tests.cases import case2d, case3d

pytestmark = pytest.mark.gpu


def _rho(shape, seed):
    rng = np.random.default_rng(seed)
    z = np.arange(shape[-1])[None, :] * 10.0
    base = 1.8 + 0.0008 * z
    return np.ascontiguousarray(base + 0.15 * rng.random(shape), np.float32)


def _desc(g, fwd=True, **kw):
    d = sw.SwPropDesc()
    d.g = g
    d.tmin, d.tmax, d.tstep = (1, g.nt, 1) if fwd else (g.nt, 1, -1)
    d.fd_scheme = sw.FD_FORWARD
    for k, v in kw.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("three_d", [False, True])
def test_rho_modeling_bitexact(ctx, oracle, three_d):
    g, vel, sou, rec, w = case3d(nt=100) if three_d else case2d(nt=300)
    rho = _rho(vel.shape, 3)
    w = sw.rho_wavelet(w, g.lsinc)
    d = _desc(g, injection=sw.INJ_SINC, extraction=sw.EXT_SINC)
    a = np.zeros((rec.shape[0], g.nt), np.float32)
    b = np.zeros_like(a)
    ctx.propagate(d, vel, sou, w, rec, a, rho=rho)
    oracle.propagate(d, vel, sou, w, rec, b, rho=rho)
    assert np.abs(b).max() > 0
    np.testing.assert_array_equal(a, b)
    # The density matters: the same run without it differs.
    c = np.zeros_like(a)
    ctx.propagate(d, vel, sou, w, rec, c)
    assert np.abs(c - a).max() > 1e-3 * np.abs(a).max()


@pytest.mark.parametrize("nz,nx", [(70, 129), (43, 20), (150, 101)])
def test_rho_modeling_ragged_tiles_bitexact(ctx, oracle, nz, nx):
    """The one-pass 2D density step on grids whose compute domain is not a
    multiple of its 64 x 32 tile, with the source near a tile corner; the
    150 x 101 grid (compute domain 170 x 121) has tiles whose gradient
    cells all lie inside the domain, which skip the per-cell tests."""
    g, vel, sou, rec, w = case2d(nz=nz, nx=nx, nt=160, seed=2)
    sou = np.array([(nz // 2) * 10.0 + 1.3, 31.0 * 10.0 if nx > 40 else 95.0, 0.0], np.float32)
    rho = _rho(vel.shape, 9)
    w = sw.rho_wavelet(w, g.lsinc)
    d = _desc(g, injection=sw.INJ_SINC, extraction=sw.EXT_SINC)
    a = np.zeros((rec.shape[0], g.nt), np.float32)
    b = np.zeros_like(a)
    ctx.propagate(d, vel, sou, w, rec, a, rho=rho)
    oracle.propagate(d, vel, sou, w, rec, b, rho=rho)
    assert np.abs(b).max() > 0
    np.testing.assert_array_equal(a, b)


def test_rho_modeling_more_tiles_than_sms_bitexact(ctx, oracle):
    """A compute domain of 720 x 421 points is 12 x 14 = 168 tiles, more
    than the device has SMs.  The source sits in tile 152 (rows 503-566,
    columns 375-406 of the compute domain), deep in the model; every
    snapshot of the whole field and the traces of a receiver line through
    the source equal the oracle's."""
    nz, nx = 700, 401
    g, vel, sou, rec, w = case2d(nz=nz, nx=nx, nt=64, seed=3, dt=5e-4)
    sou = np.array([5500.0 + 1.3, 3900.0 + 2.1, 0.0], np.float32)
    rec[:, 0] = 5450.0 + 2.3
    rho = _rho(vel.shape, 11)
    w = sw.rho_wavelet(w, g.lsinc)
    d = _desc(g, injection=sw.INJ_SINC, extraction=sw.EXT_SINC, extract_wave=1)
    out = {}
    for name, api in (("gpu", ctx), ("oracle", oracle)):
        data = np.zeros((rec.shape[0], g.nt), np.float32)
        wave = np.zeros((g.nt // g.snapi) * vel.size, np.float32)
        api.propagate(d, vel, sou, w, rec, data, wave=wave, rho=rho)
        out[name] = (data, wave)
    for a, b in zip(out["gpu"], out["oracle"]):
        assert np.abs(b).max() > 0
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("three_d", [False, True])
def test_rho_rtm_bitexact(ctx, oracle, three_d):
    """RTM_to_memory's withRho branch: forward with snapshots and the
    backward pass both on the forward-grid density operator."""
    g, vel, sou, rec, w = case3d(nt=80) if three_d else case2d(nt=200)
    rho = _rho(vel.shape, 4)
    data = (np.random.default_rng(5).standard_normal((rec.shape[0], g.nt)) * 1e-2).astype(np.float32)
    n = vel.size
    out = {}
    for name, api in (("gpu", ctx), ("oracle", oracle)):
        wave = np.zeros((g.nt // g.snapi) * n, np.float32)
        api.propagate(_desc(g, injection=sw.INJ_SINC, extract_wave=1), vel, sou, w, wave=wave,
                      rho=rho)
        im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
        api.propagate(_desc(g, False, injection=sw.INJ_SINC, imaging=sw.IMG_RTM), vel, rec, data,
                      wave=wave, image=im, illum=il, rho=rho)
        out[name] = (im, il)
    assert np.abs(out["oracle"][0]).max() > 0
    np.testing.assert_array_equal(out["gpu"][0], out["oracle"][0])
    np.testing.assert_array_equal(out["gpu"][1], out["oracle"][1])


@pytest.mark.parametrize("three_d", [False, True])
def test_rho_afwi_imaging_bitexact(ctx, oracle, three_d):
    """AFWI_to_memory's withRho branch: the backward pass on the density
    operator with Imaging_condition_AFWI_RHOVP_from_memory, whose velocity
    and density gradients (image, image2) and illumination equal the
    oracle's bit for bit."""
    g, vel, sou, rec, w = case3d(nt=80) if three_d else case2d(nt=200)
    rho = _rho(vel.shape, 7)
    data = (np.random.default_rng(8).standard_normal((rec.shape[0], g.nt)) * 1e-2).astype(np.float32)
    n = vel.size
    out = {}
    for name, api in (("gpu", ctx), ("oracle", oracle)):
        wave = np.zeros((g.nt // g.snapi) * n, np.float32)
        api.propagate(_desc(g, injection=sw.INJ_SINC, extract_wave=1), vel, sou, w, wave=wave,
                      rho=rho)
        im, im2, il = (np.zeros(n, np.float32) for _ in range(3))
        api.propagate(_desc(g, False, injection=sw.INJ_SINC, imaging=sw.IMG_AFWI_RHO), vel, rec,
                      data, wave=wave, image=im, illum=il, rho=rho, image2=im2)
        out[name] = (im, im2, il)
    for a, b in zip(out["gpu"], out["oracle"]):
        assert np.abs(b).max() > 0
        np.testing.assert_array_equal(a, b)


def test_rho_afwi_imaging_needs_density(ctx):
    g, vel, sou, rec, w = case2d(nt=40)
    n = vel.size
    wave = np.zeros((g.nt // g.snapi) * n, np.float32)
    im, im2, il = (np.zeros(n, np.float32) for _ in range(3))
    d = _desc(g, False, injection=sw.INJ_SINC, imaging=sw.IMG_AFWI_RHO)
    with pytest.raises(sw.SwaveError) as e:
        ctx.propagate(d, vel, rec, np.zeros((rec.shape[0], g.nt), np.float32), wave=wave,
                      image=im, illum=il, image2=im2)
    assert e.value.code == sw.SW_BAD_PARAM


def test_rho_rejects_the_adjoint_grid(ctx):
    g, vel, sou, rec, w = case2d(nt=50)
    d = _desc(g, injection=sw.INJ_SINC)
    d.fd_scheme = sw.FD_ADJOINT
    with pytest.raises(sw.SwaveError):
        ctx.propagate(d, vel, sou, w, rho=np.ones_like(vel))


def test_modeling_program_with_density(oracle, tmp_path):
    from seismic_gb300.build import build_cli
    built = build_cli()
    g, vel, sou, rec, w = case2d(nz=40, nx=60, nt=200)
    rho = _rho(vel.shape, 6)
    ax = {"d1": 10.0, "d2": 10.0, "o1": 0.0, "o2": 0.0}
    sep.write(str(tmp_path / "vel.H"), vel, ax)
    sep.write(str(tmp_path / "rho.H"), rho, ax)
    sep.write(str(tmp_path / "w.H"), w, {"d1": g.dt, "o1": 0.0})
    ntr = rec.shape[0]
    keys = np.zeros((ntr, 6), np.float32)
    keys[:, 0], keys[:, 1], keys[:, 4], keys[:, 5] = sou[1], rec[:, 1], sou[0], rec[:, 0]
    sep.write(str(tmp_path / "k.H"), keys)
    sep.write(str(tmp_path / "t.H"), np.zeros((ntr, g.nt), np.float32), {"d1": g.dt})
    # aperture 1000 m: the window is the whole model (clamped extraction of
    # the columns beyond it repeats the edge columns).
    params = dict(stdin=tmp_path / "w.H", vel=tmp_path / "vel.H", rho=tmp_path / "rho.H",
                  withRho=1, traces=tmp_path / "t.H", coordfile=tmp_path / "k.H", keysx=1,
                  keygx=2, keysy=3, keygy=4, keyselev=5, keygelev=6, aperture_x=0, twoD=1,
                  ntaper=g.ntaper, snapi=g.snapi, data=tmp_path / "d.H")
    r = subprocess.run(sep.command(built["Acoustic_modeling_sep.x"], **params),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    data, _ = sep.read(str(tmp_path / "d.H"))
    wv, gw = sw.shot_window(g, 0.0, 0.0, sou, rec)
    vs = sw.window_extract(g, wv, vel)
    rs = sw.window_extract(g, wv, rho)
    d = _desc(gw, injection=sw.INJ_SINC, extraction=sw.EXT_SINC)
    ref = np.zeros((ntr, g.nt), np.float32)
    oracle.propagate(d, vs, sou, sw.rho_wavelet(w, g.lsinc), rec, ref, rho=rs)
    assert np.abs(ref).max() > 0
    np.testing.assert_array_equal(data, ref)

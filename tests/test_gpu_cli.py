"""The SEP command-line programs end to end on the GPU: SEP files in, SEP
files out, against the oracle on the shot's window of the model (the
programs' windowing restated here on grid-aligned coordinates)."""
import subprocess

import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300 import sep, synth
from tests.cases import model2d, model3d

pytestmark = pytest.mark.gpu

D, DT = 10.0, 1.5e-3


@pytest.fixture(scope="module")
def built():
    from seismic_gb300.build import build_cli
    return build_cli()


def _case(tmp_path, three_d, nt=160):
    """Model 80 (x) [x 24 (y)] columns; source at x=400 (y=120), receivers
    x=300..500 (y=80..160), aperture 300 (100): window columns 25..55
    (rows 7..17)."""
    nz = 36
    if three_d:
        vel = model3d(nz, 80, 24, D, seed=4)
        rx, ry = np.meshgrid(np.arange(300.0, 501.0, 20.0), np.arange(80.0, 161.0, 40.0),
                             indexing="ij")
        rx, ry = rx.ravel(), ry.ravel()
        sou = np.array([20.3, 400.0, 120.0], np.float32)
    else:
        vel = model2d(nz, 80, D, seed=4)
        rx = np.arange(300.0, 501.0, 10.0)
        ry = np.zeros_like(rx)
        sou = np.array([20.3, 400.0, 0.0], np.float32)
    ntr = rx.size
    keys = np.zeros((ntr, 6), np.float32)
    keys[:, 0], keys[:, 1], keys[:, 2], keys[:, 3] = sou[1], rx, sou[2], ry
    keys[:, 4], keys[:, 5] = sou[0], 12.3
    rec = np.stack([np.full(ntr, 12.3), rx, ry], 1).astype(np.float32)
    w = synth.ricker(12.0, DT, nt).astype(np.float32)
    axes = {"d1": D, "d2": D, "o1": 0.0, "o2": 0.0}
    if three_d:
        axes.update({"d3": D, "o3": 0.0})
    sep.write(str(tmp_path / "vel.H"), vel, axes)
    sep.write(str(tmp_path / "w.H"), w, {"d1": DT, "o1": 0.0})
    sep.write(str(tmp_path / "keys.H"), keys)
    params = dict(stdin=tmp_path / "w.H", vel=tmp_path / "vel.H", coordfile=tmp_path / "keys.H",
                  keysx=1, keygx=2, keysy=3, keygy=4, keyselev=5, keygelev=6,
                  aperture_x=300, aperture_y=100, twoD=0 if three_d else 1, snapi=4,
                  ntaper=10, fmax=30)
    if three_d:
        win = (slice(7, 18), slice(25, 56))
        g = sw.make_genpar(nz, 31, 11, dz=D, dx=D, dy=D, ox=250.0, oy=70.0, dt=DT, nt=nt,
                           ntaper=10, lsinc=7, snapi=4, twoD=False, fmax=30.0)
    else:
        win = (slice(25, 56),)
        g = sw.make_genpar(nz, 31, 1, dz=D, dx=D, ox=250.0, dt=DT, nt=nt, ntaper=10, lsinc=7,
                           snapi=4, fmax=30.0)
    return params, g, vel, win, sou, rec, w, ntr


def _traces(tmp_path, name, arr):
    sep.write(str(tmp_path / name), arr, {"d1": DT, "o1": 0.0})
    return tmp_path / name


def _run(built, exe, params):
    r = subprocess.run(sep.command(built[exe], **params), capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stderr


@pytest.mark.parametrize("three_d", [False, True])
def test_modeling_program(built, oracle, tmp_path, three_d):
    params, g, vel, win, sou, rec, w, ntr = _case(tmp_path, three_d)
    params.update(traces=_traces(tmp_path, "t.H", np.ones((ntr, g.nt), np.float32)),
                  data=tmp_path / "d.H")
    _run(built, "Acoustic_modeling_sep.x", params)
    data, h = sep.read(str(tmp_path / "d.H"))
    assert data.shape == (ntr, g.nt)
    assert (int(h["n1"]), int(h["n2"]), float(h["d1"])) == (g.nt, ntr, pytest.approx(DT))
    ref = oracle.modeling(g, vel[win], sou, w, rec)
    assert np.abs(ref).max() > 0
    np.testing.assert_array_equal(data, ref)


@pytest.mark.parametrize("three_d", [False, True])
@pytest.mark.parametrize("lsrtm", [False, True])
def test_rtm_program(built, oracle, tmp_path, three_d, lsrtm):
    params, g, vel, win, sou, rec, w, ntr = _case(tmp_path, three_d, nt=120)
    d = (np.random.default_rng(3).standard_normal((ntr, g.nt)) * 1e-2).astype(np.float32)
    params.update(traces=_traces(tmp_path, "t.H", d), image=tmp_path / "im.H")
    if lsrtm:
        params.update(LSRTM=1)
    _run(built, "3DRTM.x", params)
    out, h = sep.read(str(tmp_path / "im.H"))
    if lsrtm:
        rim, ril = oracle.lsrtm(g, vel[win], sou, sw.born_wavelet(w, g.dt), rec, d)
    else:
        rim, ril = oracle.rtm(g, vel[win], sou, w, rec, d)
    im_full = np.zeros_like(vel)
    il_full = np.zeros_like(vel)
    im_full[win] = rim.reshape(vel[win].shape)
    il_full[win] = ril.reshape(vel[win].shape)
    assert out.shape == (2,) + vel.shape
    assert (h.get("n4") == "2") if three_d else (h["n3"] == "2")
    assert np.abs(rim).max() > 0
    np.testing.assert_array_equal(out[0], im_full)
    np.testing.assert_array_equal(out[1], il_full)


@pytest.mark.parametrize("three_d", [False, True])
def test_born_program(built, oracle, tmp_path, three_d):
    params, g, vel, win, sou, rec, w, ntr = _case(tmp_path, three_d, nt=120)
    rng = np.random.default_rng(6)
    ref = (rng.standard_normal(vel.shape) * (rng.random(vel.shape) < 0.05)).astype(np.float32)
    axes = {"d1": D, "d2": D, "o1": 0.0, "o2": 0.0}
    if three_d:
        axes.update({"d3": D, "o3": 0.0})
    sep.write(str(tmp_path / "ref.H"), ref, axes)
    params.update(traces=_traces(tmp_path, "t.H", np.zeros((ntr, g.nt), np.float32)),
                  ref=tmp_path / "ref.H", data=tmp_path / "b.H")
    _run(built, "3DBORNMOD.x", params)
    data, _ = sep.read(str(tmp_path / "b.H"))
    rd = oracle.born(g, vel[win], ref[win], sou, sw.born_wavelet(w, g.dt), rec)
    assert np.abs(rd).max() > 0
    np.testing.assert_array_equal(data, rd)

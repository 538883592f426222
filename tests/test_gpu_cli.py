"""The SEP command-line programs end to end on the GPU: SEP files in, SEP
files out, against the oracle on the shot's window of the model (the
programs' windowing restated here on grid-aligned coordinates)."""
import subprocess

import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300 import sep, synth
from tests.cases import model2d, model3d
from tests.conftest import rel_l2

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


def _cheap_lsrtm(oracle, g, vel, sou, w, rec, d):
    """CHEAP_LSRTM_to_memory: the LSRTM backward pass on the forward grid."""
    n = vel.size
    wave = np.zeros((g.nt // g.snapi) * n, np.float32)
    f = sw.SwPropDesc()
    f.g = g
    f.tmin, f.tmax, f.tstep = 1, g.nt, 1
    f.fd_scheme, f.injection, f.extract_wave = sw.FD_FORWARD, sw.INJ_SINC, 1
    oracle.propagate(f, vel, sou, w, wave=wave)
    b = sw.SwPropDesc()
    b.g = g
    b.tmin, b.tmax, b.tstep = g.nt, 1, -1
    b.fd_scheme, b.injection, b.imaging = sw.FD_FORWARD, sw.INJ_LSRTM_SINC, sw.IMG_LSRTM
    im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
    oracle.propagate(b, vel, rec, d, wave=wave, image=im, illum=il)
    return im, il


@pytest.mark.parametrize("three_d", [False, True])
@pytest.mark.parametrize("mode", ["rtm", "lsrtm", "cheap"])
def test_rtm_program(built, oracle, tmp_path, three_d, mode):
    params, g, vel, win, sou, rec, w, ntr = _case(tmp_path, three_d, nt=120)
    d = (np.random.default_rng(3).standard_normal((ntr, g.nt)) * 1e-2).astype(np.float32)
    params.update(traces=_traces(tmp_path, "t.H", d), image=tmp_path / "im.H")
    if mode != "rtm":
        params.update(LSRTM=1)
    if mode == "cheap":
        params.update(CHEAPLSRTM=1)
    _run(built, "3DRTM.x", params)
    out, h = sep.read(str(tmp_path / "im.H"))
    if mode == "lsrtm":
        rim, ril = oracle.lsrtm(g, vel[win], sou, sw.born_wavelet(w, g.dt), rec, d)
    elif mode == "cheap":
        rim, ril = _cheap_lsrtm(oracle, g, np.ascontiguousarray(vel[win]), sou,
                                sw.born_wavelet(w, g.dt), rec, d)
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
@pytest.mark.parametrize("lsrtm", [False, True])
def test_rtm_program_second_velocity(built, oracle, tmp_path, three_d, lsrtm):
    """vel2=: the backward pass and its imaging condition run on the second
    velocity (mod%vel=mod%vel2, to_disk_to_memory_RTM.f90:438-439,550-551);
    the forward pass keeps vel."""
    params, g, vel, win, sou, rec, w, ntr = _case(tmp_path, three_d, nt=120)
    vel2 = (vel * np.float32(1.04)).astype(np.float32)
    axes = {"d1": D, "d2": D, "o1": 0.0, "o2": 0.0}
    if three_d:
        axes.update({"d3": D, "o3": 0.0})
    sep.write(str(tmp_path / "vel2.H"), vel2, axes)
    d = (np.random.default_rng(3).standard_normal((ntr, g.nt)) * 1e-2).astype(np.float32)
    params.update(traces=_traces(tmp_path, "t.H", d), image=tmp_path / "im.H",
                  vel2=tmp_path / "vel2.H")
    if lsrtm:
        params.update(LSRTM=1)
    _run(built, "3DRTM.x", params)
    out, _ = sep.read(str(tmp_path / "im.H"))
    v1, v2 = np.ascontiguousarray(vel[win]), np.ascontiguousarray(vel2[win])
    wl = sw.born_wavelet(w, g.dt) if lsrtm else w
    n = v1.size
    wave = np.zeros((g.nt // g.snapi) * n, np.float32)
    f = sw.SwPropDesc()
    f.g = g
    f.tmin, f.tmax, f.tstep = 1, g.nt, 1
    f.fd_scheme, f.injection, f.extract_wave = sw.FD_FORWARD, sw.INJ_SINC, 1
    oracle.propagate(f, v1, sou, wl, wave=wave)
    b = sw.SwPropDesc()
    b.g = g
    b.tmin, b.tmax, b.tstep = g.nt, 1, -1
    if lsrtm:
        b.fd_scheme, b.injection, b.imaging = sw.FD_ADJOINT, sw.INJ_LSRTM_SINC, sw.IMG_LSRTM
    else:
        b.fd_scheme = sw.FD_FORWARD if three_d else sw.FD_ADJOINT
        b.injection, b.imaging = sw.INJ_SINC, sw.IMG_RTM
    im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
    oracle.propagate(b, v2, rec, d, wave=wave, image=im, illum=il)
    im_full, il_full = np.zeros_like(vel), np.zeros_like(vel)
    im_full[win] = im.reshape(v1.shape)
    il_full[win] = il.reshape(v1.shape)
    assert np.abs(im).max() > 0
    np.testing.assert_array_equal(out[0], im_full)
    np.testing.assert_array_equal(out[1], il_full)
    # The second velocity matters.
    ref = oracle.lsrtm(g, v1, sou, wl, rec, d) if lsrtm else oracle.rtm(g, v1, sou, w, rec, d)
    assert np.abs(ref[0] - im).max() > 1e-3 * np.abs(im).max()


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


def _survey_files(tmp_path, nt=140):
    """Three gathers on an 80-column 2D model; coordfile rows in gather
    order (the source changes between gathers)."""
    nz = 36
    vel = model2d(nz, 80, D, seed=8)
    rows, gathers = [], []
    for sx in (250.0, 400.0, 520.0):
        rx = np.arange(sx - 120.0, sx + 121.0, 20.0)
        gathers.append((sx, rx))
        for x in rx:
            rows.append([sx, x, 0.0, 0.0, 20.3, 12.3])
    keys = np.array(rows, np.float32)
    w = synth.ricker(12.0, DT, nt).astype(np.float32)
    sep.write(str(tmp_path / "vel.H"), vel, {"d1": D, "d2": D, "o1": 0.0, "o2": 0.0})
    sep.write(str(tmp_path / "w.H"), w, {"d1": DT, "o1": 0.0})
    sep.write(str(tmp_path / "keys.H"), keys)
    params = dict(stdin=tmp_path / "w.H", vel=tmp_path / "vel.H", coordfile=tmp_path / "keys.H",
                  keysx=1, keygx=2, keysy=3, keygy=4, keyselev=5, keygelev=6,
                  aperture_x=200, aperture_y=0, twoD=1, snapi=4, ntaper=10, fmax=30)
    return params, vel, w, gathers


def _gather_geometry(vel, sx, rx, nt, apx=200.0):
    """Window of one gather: centre sx (receivers symmetric about it),
    window [min(sx-120, sx-apx/2), max(sx+120, sx+apx/2)]."""
    lo = min(rx.min(), sx - apx / 2)
    hi = max(rx.max(), sx + apx / 2)
    i0, nxw = int(round(lo / D)), int(round((hi - lo) / D)) + 1
    g = sw.make_genpar(vel.shape[1], nxw, 1, dz=D, dx=D, ox=lo, dt=DT, nt=nt, ntaper=10,
                       lsinc=7, snapi=4, fmax=30.0)
    rec = np.stack([np.full(rx.size, 12.3), rx, np.zeros_like(rx)], 1).astype(np.float32)
    return g, i0, nxw, rec


def test_afwi_program_task_mod(built, oracle, tmp_path):
    params, vel, w, gathers = _survey_files(tmp_path)
    nt = w.size
    params.update(Task="MOD", data=tmp_path / "d.H")
    _run(built, "2DAFWI.x", params)
    data, h = sep.read(str(tmp_path / "d.H"))
    ntot = sum(rx.size for _, rx in gathers)
    assert data.shape == (ntot, nt) and int(h["n2"]) == ntot
    row = 0
    for sx, rx in gathers:
        g, i0, nxw, rec = _gather_geometry(vel, sx, rx, nt)
        d = sw.SwPropDesc()
        d.g = g
        d.tmin, d.tmax, d.tstep = 1, nt, 1
        d.fd_scheme, d.injection, d.extraction = sw.FD_FORWARD, sw.INJ_SINC, sw.EXT_SIMPLE_AFWI
        ref = np.zeros((rx.size, nt), np.float32)
        oracle.propagate(d, vel[i0:i0 + nxw], np.array([20.3, sx, 0.0], np.float32), w, rec, ref)
        assert np.abs(ref).max() > 0
        np.testing.assert_array_equal(data[row:row + rx.size], ref)
        row += rx.size


def test_afwi_program_task_mig(built, oracle, tmp_path):
    params, vel, w, gathers = _survey_files(tmp_path, nt=120)
    nt = w.size
    ntot = sum(rx.size for _, rx in gathers)
    obs = (np.random.default_rng(9).standard_normal((ntot, nt)) * 1e-2).astype(np.float32)
    params.update(Task="MIG", traces=_traces(tmp_path, "t.H", obs), image=tmp_path / "im.H")
    _run(built, "2DAFWI.x", params)
    img, _ = sep.read(str(tmp_path / "im.H"))
    im = np.zeros_like(vel)
    il = np.zeros_like(vel)
    row = 0
    for sx, rx in gathers:
        g, i0, nxw, rec = _gather_geometry(vel, sx, rx, nt)
        vs = vel[i0:i0 + nxw]
        sou = np.array([20.3, sx, 0.0], np.float32)
        d = sw.SwPropDesc()
        d.g = g
        d.tmin, d.tmax, d.tstep = 1, nt, 1
        d.fd_scheme, d.injection, d.extract_wave = sw.FD_FORWARD, sw.INJ_SINC, 1
        wave = np.zeros((nt // g.snapi) * vs.size, np.float32)
        oracle.propagate(d, vs, sou, w, wave=wave)
        b = sw.SwPropDesc()
        b.g = g
        b.tmin, b.tmax, b.tstep = nt, 1, -1
        b.fd_scheme, b.injection, b.imaging = sw.FD_FORWARD, sw.INJ_SIMPLE, sw.IMG_AFWI
        ims, ils = np.zeros(vs.size, np.float32), np.zeros(vs.size, np.float32)
        oracle.propagate(b, vs, rec, obs[row:row + rx.size], wave=wave, image=ims, illum=ils)
        im[i0:i0 + nxw] += ims.reshape(vs.shape)
        il[i0:i0 + nxw] += ils.reshape(vs.shape)
        row += rx.size
    r = np.sqrt(np.sum(il.astype(np.float64) ** 2) / il.size)
    norm = ((il + np.float32(il.max() / np.float32(10000))).astype(np.float64) / r).astype(np.float32)
    expect = im / norm
    assert np.abs(expect).max() > 0
    # The stacking order is the same (gather order); the FP64 RMS sum runs in
    # index order on both sides.
    np.testing.assert_allclose(img, expect, rtol=1e-6, atol=1e-6 * np.abs(expect).max())


def _inv_survey(tmp_path, built, nt=400):
    """True model with a slow blob, three gathers; observed data from the
    program's own Task=MOD; a smooth starting model."""
    nz, nx, d = 40, 90, 10.0
    z = np.arange(nz)[None, :] * d
    x = np.arange(nx)[:, None] * d
    vtrue = (1800 + 1.5 * z - 180 * np.exp(-((x - 450) ** 2 + (z - 220) ** 2) / 60.0 ** 2))
    v0 = (1800 + 1.5 * z + 0 * x)
    rows = []
    for sx in (200.0, 450.0, 700.0):
        for gx in np.arange(sx - 150.0, sx + 151.0, 20.0):
            rows.append([sx, gx, 0.0, 0.0, 20.5, 12.0])
    keys = np.array(rows, np.float32)
    w = synth.ricker(8.0, 1.5e-3, nt).astype(np.float32)
    ax = {"d1": d, "d2": d, "o1": 0.0, "o2": 0.0}
    sep.write(str(tmp_path / "vtrue.H"), vtrue.astype(np.float32), ax)
    sep.write(str(tmp_path / "v0.H"), v0.astype(np.float32), ax)
    sep.write(str(tmp_path / "w.H"), w, {"d1": 1.5e-3, "o1": 0.0})
    sep.write(str(tmp_path / "keys.H"), keys)
    common = dict(stdin=tmp_path / "w.H", coordfile=tmp_path / "keys.H", keysx=1, keygx=2,
                  keysy=3, keygy=4, keyselev=5, keygelev=6, aperture_x=100, twoD=1, snapi=4,
                  ntaper=10, fmax=20)
    _run(built, "2DAFWI.x", dict(common, vel=tmp_path / "vtrue.H", Task="MOD",
                                 data=tmp_path / "obs.H"))
    return common, v0.astype(np.float32), w, keys


_REG = dict(wantreg=1, derivdx=1, derivdz=1, log_z_plus=1, model_nrm_type="L2norm",
            compute_eps=1, ratio=5.0, wantlog=1, hinge_nrm_type="L2norm", compute_eps_log=1,
            ratio_logistic=20.0, sparse_taperx=6, sparse_taperz=4)
_NRM = {"L2norm": sw.NRM_L2, "Huber": sw.NRM_HUBER, "L1norm": sw.NRM_L1}


@pytest.mark.parametrize("nrm", [("L2norm", 0.0, None), ("Huber", 2.0, None),
                                 ("L2norm", 0.0, _REG)],
                         ids=["l2", "huber", "l2-regularised"])
def test_afwi_program_task_inv(built, oracle, tmp_path, nrm):
    """Task=INV against the oracle's restatement of the same program: the
    oracle's band-pass and mute masks, smoothing radii, its compute_fct_gdt
    (+ compute_fct_gdt_reg) and its l_bfgs driver (Inversion.f90:29-189,
    oracle.bind.l_bfgs) over its LBFGS.  The misfit history and the final
    model agree to 1e-5 relative (the gradients of the GPU and the oracle
    differ in the last bit where one FP64 norm is summed in another order,
    and the line search carries that on), the iteration count is the same
    and the misfit falls; with the L2 and Huber data norms and with the
    sparse + logistic model regularisation.  The first iteration of this
    problem takes 8-9 evaluations (the g0 scaling makes the first trial step
    overshoot), hence niter = 4 (neval = 12).  The L1 and Cauchy data norms,
    and norms whose threshold comes from the data of each evaluation, are
    left out here: the line search of this small problem stalls with them in
    the reference's algorithm as in this one; their misfit and gradient are
    compared with the oracle in test_gpu_jobs.py."""
    common, v0, w, keys = _inv_survey(tmp_path, built)
    obs, _ = sep.read(str(tmp_path / "obs.H"))
    niter = 4
    nrm_name, thresh, reg = nrm
    # A fixed Huber threshold (2 max|obs|, exact in binary) keeps the
    # residuals of this small problem in the quadratic branch; with
    # data_threshold = 0 it would follow the data of every evaluation and the
    # line search stalls.  Both branches are compared with the oracle in
    # test_gpu_jobs.py.
    thresh = round(thresh * float(np.abs(obs).max()) * 64) / 64
    _run(built, "2DAFWI.x", dict(common, vel=tmp_path / "v0.H", Task="INV",
                                 traces=tmp_path / "obs.H", niter=niter, vpmin=1500,
                                 vpmax=2600, inv=tmp_path / "inv.H",
                                 function=tmp_path / "f.H", model=tmp_path / "m.H",
                                 data_nrm_type=nrm_name, data_threshold=thresh, **(reg or {})))
    if reg:
        rdesc = sw.reg_desc(40, 90, wantreg=True, wantlog=True, derivdx=True, derivdz=True,
                            log_z_plus=True, taperz=4, taperx=6, model_nrm_type=sw.NRM_L2,
                            hinge_nrm_type=sw.NRM_L2, compute_eps=True, ratio=5.0,
                            compute_eps_log=True, ratio_log=20.0)
    else:
        rdesc = sw.reg_desc(40, 90)
    rstate = sw.SwRegState(1.0, 1.0, 0.0, 0.0)
    inv, h = sep.read(str(tmp_path / "inv.H"))
    fun, _ = sep.read(str(tmp_path / "f.H"))
    models, hm = sep.read(str(tmp_path / "m.H"))
    assert int(h["n1"]) == 40 and int(h["n2"]) == 90
    # -- the same program on the oracle -------------------------------------
    nt, dt = w.size, 1.5e-3
    g = sw.make_genpar(40, 90, 1, dz=10.0, dx=10.0, dt=dt, nt=nt, ntaper=10, lsinc=7, snapi=4,
                       fmax=20.0)
    wb = oracle.bandpass(w[None, :], dt)[0]
    ob = oracle.bandpass(obs, dt)
    desc = sw.SwFwiDesc()
    desc.g = g
    desc.aperture_x, desc.aperture_y, desc.illu_pow = 100.0, 0.0, 1.0
    # Init_SmoothingParam (Smoothing.f90:36-85) with the program's defaults.
    velref = np.float32((v0.max() - v0.min()) / np.float32(2) + v0.min())
    freqref = np.float32(0.0 + (20.0 - 0.0) / 2)
    wave = np.float32(0.5) * velref / freqref
    r = int((wave / np.float32(10.0) + np.float32(1.5)) / np.float32(2))
    desc.smooth_rect1, desc.smooth_rect2, desc.smooth_rect3 = r, r, int((0 + 1.5) / 2)
    desc.smooth_doz = desc.smooth_dox = int(not wave <= 10.0)
    desc.smooth_doy = 0
    desc.dat_nrm_type = _NRM[nrm_name]
    desc.dat_thresh = thresh
    shots, row = [], 0
    for sx in (200.0, 450.0, 700.0):
        sel = keys[:, 0] == sx
        rec = np.stack([keys[sel, 5], keys[sel, 1], keys[sel, 3]], 1).astype(np.float32)
        sou = np.array([20.5, sx, 0.0], np.float32)
        shots.append({"sou": sou, "rec": rec, "dobs": ob[row:row + rec.shape[0]],
                      "mute": oracle.mute_mask(nt, dt, sou, rec)})
        row += rec.shape[0]

    def fctgdt(x, eval_):
        f, grad, _ = oracle.fwi_fct_gdt(desc, x.reshape(v0.shape), wb, shots)
        return oracle.fwi_regularize(rdesc, rstate, eval_, x, f, grad.ravel())

    x, fhist, omodels = oracle.l_bfgs(fctgdt, v0, niter, 3 * niter, 1500.0, 2600.0,
                                      vpinit=v0.astype(np.float64))
    # 2DAFWI's final FREEZE_X and mask (all ones here) of the model it writes.
    x = np.minimum(np.float32(2600), np.maximum(np.float32(1500), x))
    it = len(omodels)
    assert it >= 1 and fun.size == fhist.size
    assert models.size == it * 40 * 90 and int(hm["n4"]) == it
    assert rel_l2(fun, fhist) < 1e-5, (fun, fhist)
    dm, rdm = inv.ravel() - v0.ravel(), x - v0.ravel()
    assert np.abs(rdm).max() > 1.0                    # the model moved
    assert rel_l2(dm, rdm) < 1e-5
    assert fun[-1] < fun[0]


def _lbfgs_program_loop(built, oracle, tmp_path, lbfgs_type, nsteps=40):
    """Drives L_BFGS.x as the reference's workflow does: write Model,
    Function and Gradient, run the program in the state directory, rename
    its *Out.dat files to the names it reads, evaluate at the model it wrote,
    repeat.  The same loop on the oracle (state kept in memory, the model
    rounded to FP32 between calls as the SEP files do)."""
    import os
    rng = np.random.default_rng(21)
    n1, n2, n3 = 30, 20, 2                 # n3 < 5: a parameter axis (nparams = 2)
    n = n1 * n2 * n3
    t = np.concatenate([rng.uniform(1600.0, 2400.0, n // 2),
                        rng.uniform(2100.0, 2500.0, n // 2)]).astype(np.float64)
    a = rng.uniform(0.5, 2.0, n)
    xmin, xmax = [1500.0, 2000.0], [2500.0, 2600.0]
    x0 = np.full(n, 2000.0, np.float32)
    run = tmp_path / "state"
    run.mkdir()
    shape = (n3, n2, n1)
    sep.write(str(run / "init.H"), x0.reshape(shape))
    sep.write(str(run / "mod.H"), x0.reshape(shape))
    params = dict(Model=run / "mod.H", Function=run / "fct.H", Gradient=run / "grad.H",
                  lbfgs_type=lbfgs_type, bound_type=1, stp1_opt=1)
    if lbfgs_type == 1:
        params.update(Initial_Model=run / "init.H", xmin=",".join(map(str, xmin)),
                      xmax=",".join(map(str, xmax)))
    models, flags = [], []
    for _ in range(nsteps):
        x, _ = sep.read(str(run / "mod.H"))
        x = x.ravel().astype(np.float64)
        r = x - t
        sep.write(str(run / "fct.H"), np.array([0.5 * np.sum(a * r * r)], np.float32))
        sep.write(str(run / "grad.H"), (a * r).astype(np.float32).reshape(shape))
        res = subprocess.run(sep.command(built["L_BFGS.x"], **params), capture_output=True,
                             text=True, timeout=300, cwd=run)
        assert res.returncode == 0, res.stderr
        for nm in ("Diag", "Iflag", "Info", "LbfgsDat", "McsrchDat", "WorkArray"):
            os.replace(run / f"{nm}Out.dat", run / f"{nm}.dat")
        iflag = int((run / "Iflag.dat").read_text().split()[0])
        m, _ = sep.read(str(run / "mod.H"))
        models.append(m.ravel().copy())
        flags.append(iflag)
        if iflag <= 0:
            break
    # The oracle over the same FP32 function / gradient / model round trips.
    import seismic_gb300 as sw
    d, keep = sw.lbfgs_oc_desc(n, 5, n3, xmin, xmax, lbfgs_type, 1, 1)
    w = np.zeros(n * 11 + 10)
    diag = np.zeros(n)
    st = sw.SwLbfgsOcState()
    iflag, rmodels, rflags = 0, [], []
    x = x0.astype(np.float64)
    for _ in range(len(models)):
        r = x - t
        f = float(np.float32(0.5 * np.sum(a * r * r)))
        g = (a * r).astype(np.float32).astype(np.float64)
        iflag, _ = oracle.lbfgs_oc_step(d, x, f, g, w, diag, st, iflag, 0)
        x = x.astype(np.float32).astype(np.float64)
        rmodels.append(x.astype(np.float32))
        rflags.append(iflag)
        if iflag <= 0:
            break
    return models, flags, rmodels, rflags, t


@pytest.mark.parametrize("lbfgs_type", [1, 0])
def test_lbfgs_program_multi_invocation(built, oracle, tmp_path, lbfgs_type):
    """L_BFGS.x (progs/inversion/L_BFGS.f90) run once per function
    evaluation with its state in the reference's files (Iflag, Info, Diag,
    WorkArray, LbfgsDat, McsrchDat) against the oracle's LBFGSOC / LBFGSOLD
    keeping the state in memory: the same iflag sequence, the same models
    to FP32 rounding, the model approaching the minimum and, for
    lbfgs_type 1, every model inside the per-parameter bounds."""
    models, flags, rmodels, rflags, t = _lbfgs_program_loop(built, oracle, tmp_path, lbfgs_type)
    assert flags == rflags and len(models) >= 10
    for u, v in zip(models, rmodels):
        assert np.abs(u - v).max() <= 1e-5 * np.abs(v).max()
    first = np.abs(np.full_like(t, 2000.0) - t).max()
    assert np.abs(models[-1] - t).max() < 0.05 * first
    if lbfgs_type == 1:
        half = t.size // 2
        for m in models:
            assert m[:half].min() >= 1500.0 and m[:half].max() <= 2500.0
            assert m[half:].min() >= 2000.0 and m[half:].max() <= 2600.0

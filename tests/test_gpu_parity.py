"""GPU-vs-oracle parity through the C-ABI (libswave.so).

The CUDA kernels evaluate every expression in the reference's order with
FMA contraction disabled, so the bar for FP32 wavefields and traces is
bit-exact equality with the oracle; the benchmark spec's tolerance (1e-5 relative
L2) is asserted as well so that a failure reports both.
"""
import numpy as np
import pytest

import seismic_gb300 as sw
from tests.cases import case2d, case3d
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5   # spec tolerance, relative L2


def _desc(g, fwd=True, **kw):
    d = sw.SwPropDesc()
    d.g = g
    if fwd:
        d.tmin, d.tmax, d.tstep = 1, g.nt, 1
    else:
        d.tmin, d.tmax, d.tstep = g.nt, 1, -1
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_modeling_2d_bitexact(ctx, oracle):
    g, vel, sou, rec, w = case2d(nt=400)
    data, fu = ctx.modeling(g, vel, sou, w, rec, final_u2=True)
    ref, rfu = oracle.modeling(g, vel, sou, w, rec, final_u2=True)
    assert np.abs(ref).max() > 0
    assert rel_l2(data, ref) < TOL
    assert rel_l2(fu, rfu) < TOL
    np.testing.assert_array_equal(data, ref)
    np.testing.assert_array_equal(fu, rfu)


def test_modeling_3d_bitexact(ctx, oracle):
    g, vel, sou, rec, w = case3d(nt=100)
    data, fu = ctx.modeling(g, vel, sou, w, rec, final_u2=True)
    ref, rfu = oracle.modeling(g, vel, sou, w, rec, final_u2=True)
    assert np.abs(ref).max() > 0
    assert rel_l2(data, ref) < TOL
    np.testing.assert_array_equal(data, ref)
    np.testing.assert_array_equal(fu, rfu)


def test_config1_modeling(ctx, oracle):
    """Config 1 at full size: 201x401, 10 m, 2000 steps, ntaper 40."""
    from seismic_gb300 import synth
    c = synth.config1()
    data, fu = ctx.modeling(c["g"], c["vel"], c["sou"], c["wavelet"], c["rec"], final_u2=True)
    ref, rfu = oracle.modeling(c["g"], c["vel"], c["sou"], c["wavelet"], c["rec"], final_u2=True)
    assert data.shape == (401, 2000)
    assert rel_l2(data, ref) < TOL
    assert rel_l2(fu, rfu) < TOL
    np.testing.assert_array_equal(data, ref)


@pytest.mark.parametrize("twoD", [True, False])
def test_rtm_bitexact(ctx, oracle, twoD):
    g, vel, sou, rec, w = case2d(nt=240) if twoD else case3d(nt=80)
    data = oracle.modeling(g, vel, sou, w, rec)
    im, il = ctx.rtm(g, vel, sou, w, rec, data)
    rim, ril = oracle.rtm(g, vel, sou, w, rec, data)
    assert np.abs(rim).max() > 0
    assert rel_l2(im, rim) < TOL and rel_l2(il, ril) < TOL
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


@pytest.mark.parametrize("nz", [32, 28])
def test_rtm_lsrtm_3d_vector_snapshot_path(ctx, oracle, nz):
    """3D RTM and LSRTM where every column's snapshot rows are 16-byte
    aligned (nz = 32, 28 with an 8-cell taper: the 16-byte snapshot and
    imaging accesses of the step kernel) against the oracle, bit for bit;
    case3d's nz = 30 mixes aligned and unaligned columns."""
    g, vel, sou, rec, w = case3d(nz=nz, nt=80)
    data = oracle.modeling(g, vel, sou, w, rec)
    im, il = ctx.rtm(g, vel, sou, w, rec, data)
    rim, ril = oracle.rtm(g, vel, sou, w, rec, data)
    assert np.abs(rim).max() > 0
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)
    w2 = sw.born_wavelet(w, g.dt)
    im, il = ctx.lsrtm(g, vel, sou, w2, rec, data)
    rim, ril = oracle.lsrtm(g, vel, sou, w2, rec, data)
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


@pytest.mark.parametrize("twoD", [True, False])
def test_born_lsrtm_bitexact(ctx, oracle, twoD):
    g, vel, sou, rec, w = case2d(nt=240) if twoD else case3d(nt=80)
    w2 = sw.born_wavelet(w, g.dt)
    rng = np.random.default_rng(5)
    ref = (rng.standard_normal(vel.shape) * (rng.random(vel.shape) < 0.05)).astype(np.float32)
    data = ctx.born(g, vel, ref, sou, w2, rec)
    rdata = oracle.born(g, vel, ref, sou, w2, rec)
    assert np.abs(rdata).max() > 0
    assert rel_l2(data, rdata) < TOL
    np.testing.assert_array_equal(data, rdata)
    im, il = ctx.lsrtm(g, vel, sou, w2, rec, rdata)
    rim, ril = oracle.lsrtm(g, vel, sou, w2, rec, rdata)
    assert rel_l2(im, rim) < TOL
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


@pytest.mark.parametrize("inj,ext,fd", [
    (sw.INJ_SINC, sw.EXT_SINC_AFWI, sw.FD_FORWARD),
    (sw.INJ_SIMPLE, sw.EXT_SIMPLE_AFWI, sw.FD_ADJOINT),
    (sw.INJ_LSRTM_SINC, sw.EXT_LSRTM_SINC, sw.FD_FORWARD),
])
def test_propagate_options(ctx, oracle, inj, ext, fd):
    g, vel, sou, rec, w = case2d(nt=150)
    d = _desc(g, True, fd_scheme=fd, injection=inj, extraction=ext, extract_wave=1)
    ntsnap = g.nt // g.snapi
    tr0 = np.random.default_rng(1).standard_normal((rec.shape[0], g.nt)).astype(np.float32)
    a_tr, b_tr = tr0.copy(), tr0.copy()
    a_w = np.zeros(ntsnap * g.nz * g.nx, np.float32)
    b_w = a_w.copy()
    ctx.propagate(d, vel, sou, w, rec, a_tr, wave=a_w)
    oracle.propagate(d, vel, sou, w, rec, b_tr, wave=b_w)
    np.testing.assert_array_equal(a_tr, b_tr)
    np.testing.assert_array_equal(a_w, b_w)


def test_afwi_imaging_backward(ctx, oracle):
    """AGRAD-style backward propagation with the AFWI imaging condition."""
    g, vel, sou, rec, w = case2d(nt=160)
    ntsnap = g.nt // g.snapi
    rng = np.random.default_rng(2)
    wave = rng.standard_normal(ntsnap * g.nz * g.nx).astype(np.float32)
    adj = rng.standard_normal((rec.shape[0], g.nt)).astype(np.float32)
    d = _desc(g, False, fd_scheme=sw.FD_FORWARD, injection=sw.INJ_SIMPLE, imaging=sw.IMG_AFWI)
    n = g.nz * g.nx
    a_im, a_il = np.zeros(n, np.float32), np.zeros(n, np.float32)
    b_im, b_il = a_im.copy(), a_il.copy()
    ctx.propagate(d, vel, rec, adj, wave=wave.copy(), image=a_im, illum=a_il)
    oracle.propagate(d, vel, rec, adj, wave=wave.copy(), image=b_im, illum=b_il)
    np.testing.assert_array_equal(a_im, b_im)
    np.testing.assert_array_equal(a_il, b_il)


def test_bad_params_are_rejected(ctx):
    g, vel, sou, rec, w = case2d(nt=10)
    g.lsinc = 8
    with pytest.raises(sw.SwaveError) as e:
        ctx.modeling(g, vel, sou, w, rec)
    assert e.value.code == sw.SW_BAD_PARAM
    g, vel, sou, rec, w = case2d(nt=10)
    g.surf_type = -1
    with pytest.raises(sw.SwaveError) as e:
        ctx.modeling(g, vel, sou, w, rec)
    assert e.value.code == sw.SW_BAD_PARAM
    g, vel, sou, rec, w = case2d(nt=10)
    bad = sou.copy()
    bad[1] = -1000.0   # footprint outside the compute domain
    with pytest.raises(sw.SwaveError) as e:
        ctx.modeling(g, vel, bad, w, rec)
    assert e.value.code == sw.SW_BAD_PARAM


def test_linearity_scaling(ctx):
    """Modelling is linear in the wavelet.  Doubling is exact in FP32 except
    where early-time values underflow into subnormals, so the check is a
    relative one."""
    g, vel, sou, rec, w = case2d(nt=200)
    a = ctx.modeling(g, vel, sou, w, rec)
    b = ctx.modeling(g, vel, sou, 2 * w, rec)
    assert rel_l2(b, 2 * a) < 1e-6


@pytest.mark.parametrize("three_d", [False, True])
def test_born_lsrtm_dot_test_rigid(oracle, three_d):
    """Exact-adjoint mode (sw_ctx_set_boundary(ctx, 1)): the GPU Born and
    LSRTM operators pass the dot-product test to 1e-5 in FP32 and match the
    oracle's rigid-boundary runs bit for bit."""
    from tests.cases import case2d, case3d
    if three_d:
        g, vel, sou, rec, w = case3d(nt=100, snapi=2)
    else:
        g, vel, sou, rec, w = case2d(nz=50, nx=70, nt=400, seed=2, snapi=4)
    rng = np.random.default_rng(35)
    m = rng.standard_normal(vel.shape).astype(np.float32)
    d = rng.standard_normal((rec.shape[0], g.nt)).astype(np.float32)
    c = sw.Context(0)
    try:
        c.set_boundary(1)
        lm = c.born(g, vel, m, sou, w, rec)
        ltd, _ = c.lsrtm(g, vel, sou, w, rec, d)
    finally:
        c.close()
    a = float(np.sum(lm.astype(np.float64) * d))
    b = float(np.sum(m.ravel().astype(np.float64) * ltd.ravel()))
    assert abs(a - b) <= 1e-5 * max(abs(a), abs(b))
    oracle.set_rigid(True)
    try:
        rlm = oracle.born(g, vel, m, sou, w, rec)
        rltd, _ = oracle.lsrtm(g, vel, sou, w, rec, d)
    finally:
        oracle.set_rigid(False)
    np.testing.assert_array_equal(lm, rlm)
    np.testing.assert_array_equal(ltd, rltd)


@pytest.mark.parametrize("kernel", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("fd", [sw.FD_FORWARD, sw.FD_ADJOINT])
@pytest.mark.parametrize("imaging", [sw.IMG_RTM, sw.IMG_LSRTM, sw.IMG_AFWI])
def test_backward_imaging_every_grid_and_kernel(oracle, kernel, fd, imaging):
    """Every imaging condition on either stencil grid (the CHEAP_LSRTM
    backward pass images on the forward grid) with every 2D step kernel."""
    g, vel, sou, rec, w = case2d(nt=120)
    ntsnap = g.nt // g.snapi
    rng = np.random.default_rng(7)
    wave = rng.standard_normal(ntsnap * g.nz * g.nx).astype(np.float32)
    adj = rng.standard_normal((rec.shape[0], g.nt)).astype(np.float32)
    inj = sw.INJ_SIMPLE if imaging == sw.IMG_AFWI else (
        sw.INJ_LSRTM_SINC if imaging == sw.IMG_LSRTM else sw.INJ_SINC)
    d = _desc(g, False, fd_scheme=fd, injection=inj, imaging=imaging)
    n = g.nz * g.nx
    a_im, a_il = np.zeros(n, np.float32), np.zeros(n, np.float32)
    b_im, b_il = a_im.copy(), a_il.copy()
    c = sw.Context(0)
    try:
        c.set_tuning(step_kernel=kernel)
        c.propagate(d, vel, rec, adj, wave=wave.copy(), image=a_im, illum=a_il)
    finally:
        c.close()
    oracle.propagate(d, vel, rec, adj, wave=wave.copy(), image=b_im, illum=b_il)
    assert np.abs(b_im).max() > 0
    np.testing.assert_array_equal(a_im, b_im)
    np.testing.assert_array_equal(a_il, b_il)


@pytest.mark.parametrize("nt", [400, 401])
@pytest.mark.parametrize("rigid", [0, 1])
@pytest.mark.parametrize("shape", [(60, 80), (45, 130), (130, 45), (30, 36)])
def test_modeling_two_step_kernel(oracle, nt, rigid, shape):
    """The two-step tile kernel (step_kernel 4: steps s and s + 1 in one
    launch, step A over the tile grown by 4 cells, Higdon edges of both
    steps in the tile): traces and the final wavefield bit-exact with the
    oracle, for an even and an odd number of steps, with the Higdon and the
    rigid boundary, on grids with one and several tiles along each axis."""
    nz, nx = shape
    g, vel, sou, rec, w = case2d(nz=nz, nx=nx, nt=nt)
    c = sw.Context(0)
    try:
        c.set_tuning(step_kernel=4)
        c.set_boundary(rigid)
        data, fu = c.modeling(g, vel, sou, w, rec, final_u2=True)
    finally:
        c.close()
    oracle.set_rigid(bool(rigid))
    try:
        ref, rfu = oracle.modeling(g, vel, sou, w, rec, final_u2=True)
    finally:
        oracle.set_rigid(False)
    assert np.abs(ref).max() > 0
    np.testing.assert_array_equal(data, ref)
    np.testing.assert_array_equal(fu, rfu)


@pytest.mark.parametrize("nz", [30, 20])
def test_modeling_3d_partial_last_tile(ctx, oracle, nz):
    """3D modelling whose last 32-row tile of the pipelined 3D kernel owns
    14 rows (nz 30) or 4 rows (nz 20), the second inside the Higdon bottom
    edge zone: traces and final wavefield bit-exact."""
    g, vel, sou, rec, w = case3d(nz=nz, nt=100)
    data, fu = ctx.modeling(g, vel, sou, w, rec, final_u2=True)
    ref, rfu = oracle.modeling(g, vel, sou, w, rec, final_u2=True)
    assert np.abs(ref).max() > 0
    np.testing.assert_array_equal(data, ref)
    np.testing.assert_array_equal(fu, rfu)

"""The oracle's 2DAFWI model regularisation (compute_fct_gdt_reg,
progs/afwi/compute_function_gradient.f90:98-206, with
libs/libwave/Sparse_regularization.f90 and the helix filters of
libs/libflt/helicon.f90) against an independent numpy restatement, and the
eps / threshold state it keeps between evaluations."""
import numpy as np
import pytest

import seismic_gb300 as sw
from tests.test_oracle_norms import _fct, _gdt

F = np.float32


def _pad(a, tz, tx, ty):
    """add_taper forw: edge replication, Fortran (z fastest) order."""
    return np.pad(a, ((ty, ty), (tx, tx), (tz, tz)), mode="edge")


def _helix(x, lag, adj):
    y = (F(0) + x).astype(F)
    if adj:
        y[:-lag] = y[:-lag] + x[lag:] * F(-1)
    else:
        y[lag:] = y[lag:] + x[:-lag] * F(-1)
    return y


def _pass(a_shape, vel, zw, lag, mode, ntype, thresh, t):
    """One Compute_f_g; vel/zw are (ny, nx, nz) arrays.  Returns (f, g, thresh)."""
    ny, nx, nz = a_shape
    tz, tx, ty = t
    vt = _pad(vel, tz, tx, ty).ravel()
    zwt = _pad(zw, tz, tx, ty).ravel() if zw is not None else np.ones_like(vt)
    rm = _helix(vt, lag, False)
    if mode == 2:
        mask = np.where(rm <= 0, F(1), F(0)).astype(F)
        rm = (rm * mask * zwt).astype(F)
    else:
        mask = np.where(rm <= 0, F(0), F(1)).astype(F) if mode == 1 else np.ones_like(rm)
        rm = (rm * zwt * mask).astype(F)
    shp = (ny + 2 * ty, nx + 2 * tx, nz + 2 * tz)
    inner = lambda v: v.reshape(shp)[ty:ty + ny, tx:tx + nx, tz:tz + nz]
    gt = (F(0) + inner(rm)).astype(F)
    f, thresh = _fct(ntype, gt.ravel()[:nz * nx], thresh)
    ng = shp[1] * shp[2]
    rm[:ng] = _gdt(ntype, rm[:ng], thresh) if ntype != sw.NRM_L2 else rm[:ng]
    rm = (mask * rm * zwt).astype(F) if mode == 2 else (rm * zwt * mask).astype(F)
    rt = _helix(rm, lag, True)
    return f, (F(0) + inner(rt)).astype(F), thresh


def _reference(d, st, eval_, vel, f, grad, vpmask, zw):
    """compute_fct_gdt_reg restated over numpy; st is a dict, updated."""
    nz, nx, ny = d["nz"], d["nx"], d["ny"]
    t = (d["tz"], d["tx"], d["ty"] if ny != 1 else 0)
    shape = (ny, nx, nz)
    v = vel.reshape(shape)
    z = zw.reshape(shape) if zw is not None else None
    nzt = nz + 2 * t[0]
    scaling = float(nx * ny * nz)
    grad = grad.copy()
    ftmp = ftmp1 = 0.0
    if d["compute_eps"] and eval_ == 0:
        st["eps"] = F(0)
    if d["wantreg"]:
        g = np.zeros(shape, F)
        passes = []
        if d["derivdx"]:
            passes.append((nzt, 0))
        if d["derivdz"]:
            passes.append((1, 1 if d["log_z_plus"] else 0))
        if ny != 1 and d["derivdy"]:
            passes.append((nzt, 0))
        for lag, mode in passes:
            fp, gp, st["mod_thresh"] = _pass(shape, v, z, lag, mode, d["mtype"],
                                             st["mod_thresh"], t)
            ftmp += fp
            g = (g + gp).astype(F)
        ftmp /= scaling
        g = (g / F(scaling)).astype(F)
        if d["compute_eps"] and eval_ == 0:
            st["eps"] = F(0) if d["ratio"] == 0 else F(abs(f / (float(F(d["ratio"])) * ftmp)))
        grad = (grad - g.ravel() * st["eps"]).astype(F)
    else:
        st["eps"] = F(0)
    if d["wantlog"]:
        fp, gp, st["hin_thresh"] = _pass(shape, v, z, 1, 2, d["htype"], st["hin_thresh"], t)
        ftmp1 = fp / scaling
        g = (gp / F(scaling)).astype(F)
        grad = (grad - g.ravel() * st["eps_log"]).astype(F)
    else:
        st["eps_log"] = F(0)
    if vpmask is not None:
        grad = (grad * vpmask).astype(F)
    return f + ftmp * float(st["eps"]) + ftmp1 * float(st["eps_log"]), grad


def _model(nz=9, nx=11, ny=1, seed=0):
    rng = np.random.default_rng(seed)
    z = np.arange(nz, dtype=np.float64)[None, None, :]
    v = 1800 + 25 * z + 40 * rng.standard_normal((ny, nx, nz))
    return v.astype(F).ravel()


CASES = {
    "dx_l2": dict(wantreg=1, derivdx=1, mtype=sw.NRM_L2),
    "dz_cauchy": dict(wantreg=1, derivdz=1, mtype=sw.NRM_CAUCHY),
    "dxdz_huber_hinge": dict(wantreg=1, derivdx=1, derivdz=1, log_z_plus=1, mtype=sw.NRM_HUBER),
    "dxdz_l1": dict(wantreg=1, derivdx=1, derivdz=1, mtype=sw.NRM_L1),
    "logistic_l2": dict(wantlog=1, htype=sw.NRM_L2),
    "both_hyperbolic": dict(wantreg=1, wantlog=1, derivdz=1, mtype=sw.NRM_HYPERBOLIC,
                            htype=sw.NRM_HUBER),
}


def _desc(case, nz, nx, ny, tz=3, tx=4, ty=0):
    c = dict(nz=nz, nx=nx, ny=ny, tz=tz, tx=tx, ty=ty, wantreg=0, wantlog=0, derivdx=0,
             derivdy=0, derivdz=0, log_z_plus=0, mtype=sw.NRM_CAUCHY, htype=sw.NRM_L2,
             compute_eps=0, ratio=10.0)
    c.update(CASES[case])
    d = sw.reg_desc(nz, nx, ny, wantreg=c["wantreg"], wantlog=c["wantlog"],
                    derivdx=c["derivdx"], derivdy=c["derivdy"], derivdz=c["derivdz"],
                    log_z_plus=c["log_z_plus"], taperz=tz, taperx=tx, tapery=ty,
                    model_nrm_type=c["mtype"], hinge_nrm_type=c["htype"])
    return c, d


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_regularize_matches_restatement(oracle, case):
    nz, nx = 9, 11
    c, d = _desc(case, nz, nx, 1)
    vel = _model(nz, nx)
    rng = np.random.default_rng(2)
    grad = rng.standard_normal(vel.size).astype(F)
    mask = (rng.random(vel.size) > 0.1).astype(F) * F(2)
    zw = (0.5 + rng.random(vel.size)).astype(F)
    st = sw.SwRegState(1.0, 0.7, 0.0, 0.0)
    f, g = oracle.fwi_regularize(d, st, 3, vel, 1.25, grad, vpmask=mask, zweight=zw)
    rst = {"eps": F(1.0), "eps_log": F(0.7), "mod_thresh": F(0), "hin_thresh": F(0)}
    rf, rg = _reference(c, rst, 3, vel, 1.25, grad, mask, zw)
    tol = 1e-6 if sw.NRM_CAUCHY in (c["mtype"],) and c["wantreg"] else 0.0
    np.testing.assert_array_equal(g, rg)
    assert abs(f - rf) <= tol * abs(rf)
    assert st.mod_thresh == rst["mod_thresh"] and st.hin_thresh == rst["hin_thresh"]
    assert f != 1.25


def test_no_regularisation_only_masks(oracle):
    d = sw.reg_desc(5, 6)
    rng = np.random.default_rng(1)
    grad = rng.standard_normal(30).astype(F)
    mask = np.array([0, 1, 2] * 10, F)
    st = sw.SwRegState(1.0, 1.0, 0.0, 0.0)
    f, g = oracle.fwi_regularize(d, st, 0, _model(5, 6), 2.0, grad, vpmask=mask)
    assert f == 2.0
    np.testing.assert_array_equal(g, grad * mask)
    assert st.eps == 0 and st.eps_log == 0


def test_eps_from_ratio_at_the_first_evaluation_only(oracle):
    """compute_eps: eps = |f / (ratio * ftmp)| at evaluation 0, kept after."""
    nz, nx = 8, 10
    d = sw.reg_desc(nz, nx, wantreg=True, derivdz=True, model_nrm_type=sw.NRM_L2,
                    compute_eps=True, ratio=4.0)
    vel = _model(nz, nx)
    st = sw.SwRegState(0.0, 0.0, 0.0, 0.0)
    grad = np.zeros(vel.size, F)
    f0 = 3.0
    f, _ = oracle.fwi_regularize(d, st, 0, vel, f0, grad)
    # The regularisation adds f0 / ratio at evaluation 0.
    assert abs(f - (f0 + f0 / 4.0)) < 1e-6
    eps0 = st.eps
    f, _ = oracle.fwi_regularize(d, st, 1, vel * F(1.01), 9.0, grad)
    assert st.eps == eps0


def test_threshold_is_set_once_and_kept(oracle):
    """reg_threshold = 0: the first fct_compute sets it to max|.|, and the
    state keeps it for the following passes and evaluations."""
    nz, nx = 8, 10
    d = sw.reg_desc(nz, nx, wantreg=True, derivdx=True, derivdz=True,
                    model_nrm_type=sw.NRM_HUBER)
    vel = _model(nz, nx)
    st = sw.SwRegState(1.0, 0.0, 0.0, 0.0)
    oracle.fwi_regularize(d, st, 0, vel, 0.0, np.zeros(vel.size, F))
    t0 = st.mod_thresh
    assert t0 > 0
    oracle.fwi_regularize(d, st, 1, vel * F(3), 0.0, np.zeros(vel.size, F))
    assert st.mod_thresh == t0


def test_logistic_penalises_only_velocity_decreasing_with_depth(oracle):
    nz, nx = 8, 6
    z = np.arange(nz, dtype=F)[None, :]
    up = np.broadcast_to(1500 + 30 * z, (nx, nz)).astype(F).ravel()
    down = np.broadcast_to(1500 - 30 * z, (nx, nz)).astype(F).ravel()
    st = sw.SwRegState(0.0, 1.0, 0.0, 0.0)
    # With the z taper the helix wrap (bottom of one column to the top of the
    # next) falls in the pad: a model increasing with depth costs nothing.
    d = sw.reg_desc(nz, nx, wantlog=True, hinge_nrm_type=sw.NRM_L2, taperz=2, taperx=0)
    f, g = oracle.fwi_regularize(d, st, 1, up, 0.0, np.zeros(up.size, F))
    assert f == 0 and not g.any()
    f, g = oracle.fwi_regularize(d, st, 1, down, 0.0, np.zeros(up.size, F))
    assert abs(f - 30.0 ** 2 / 2 * (nz - 1) * nx / up.size) < 1e-9 * f
    assert g.any()
    # Without it the wrap sample of every column but the first is negative.
    d = sw.reg_desc(nz, nx, wantlog=True, hinge_nrm_type=sw.NRM_L2, taperz=0, taperx=0)
    f, _ = oracle.fwi_regularize(d, st, 1, up, 0.0, np.zeros(up.size, F))
    assert abs(f - (30.0 * (nz - 1)) ** 2 / 2 * (nx - 1) / up.size) < 1e-9 * f


def test_3d_y_pass_uses_the_x_filter(oracle):
    """derivdy in 3D repeats the x pass (helicon2_mod_lop carries the x
    filter): dx+dy equals twice dx."""
    nz, nx, ny = 5, 6, 4
    vel = _model(nz, nx, ny)
    st = sw.SwRegState(1.0, 0.0, 0.0, 0.0)
    dx = sw.reg_desc(nz, nx, ny, wantreg=True, derivdx=True, model_nrm_type=sw.NRM_L2,
                     tapery=2)
    dxy = sw.reg_desc(nz, nx, ny, wantreg=True, derivdx=True, derivdy=True,
                      model_nrm_type=sw.NRM_L2, tapery=2)
    f1, g1 = oracle.fwi_regularize(dx, st, 1, vel, 0.0, np.zeros(vel.size, F))
    f2, g2 = oracle.fwi_regularize(dxy, st, 1, vel, 0.0, np.zeros(vel.size, F))
    assert f2 == 2 * f1
    np.testing.assert_array_equal(g2, (g1 * F(2)).astype(F))

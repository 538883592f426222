"""sw_fwi_regularize (compute_fct_gdt_reg's sparse and logistic
regularisation, progs/afwi/compute_function_gradient.f90:98-206) against the
oracle through the C-ABI: gradients and state bit-exact, the misfit bit-exact
except the FP32 log of the Cauchy norm (CUDA's logf against the C
library's, 1e-6)."""
import numpy as np
import pytest

import seismic_gb300 as sw
from tests.test_oracle_regularize import CASES, _desc, _model

pytestmark = pytest.mark.gpu
F = np.float32


def _both(ctx, oracle, d, st_args, eval_, vel, f, grad, mask=None, zw=None):
    sg, so = sw.SwRegState(*st_args), sw.SwRegState(*st_args)
    fg, gg = ctx.fwi_regularize(d, sg, eval_, vel, f, grad, vpmask=mask, zweight=zw)
    fo, go = oracle.fwi_regularize(d, so, eval_, vel, f, grad, vpmask=mask, zweight=zw)
    return (fg, gg, sg), (fo, go, so)


def _check(a, b, cauchy):
    (fg, gg, sg), (fo, go, so) = a, b
    np.testing.assert_array_equal(gg, go)
    assert (sg.eps, sg.eps_log, sg.mod_thresh, sg.hin_thresh) == \
        (so.eps, so.eps_log, so.mod_thresh, so.hin_thresh)
    if cauchy:
        assert abs(fg - fo) <= 1e-6 * abs(fo)
    else:
        assert fg == fo


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("size", [(9, 11), (301, 517)])
def test_regularize_matches_oracle(ctx, oracle, case, size):
    nz, nx = size
    c, d = _desc(case, nz, nx, 1, tz=10, tx=10)
    vel = _model(nz, nx)
    rng = np.random.default_rng(4)
    grad = rng.standard_normal(vel.size).astype(F)
    mask = (rng.random(vel.size) > 0.1).astype(F)
    zw = (0.5 + rng.random(vel.size)).astype(F)
    a, b = _both(ctx, oracle, d, (1.0, 0.7, 0.0, 0.0), 2, vel, 1.25, grad, mask, zw)
    _check(a, b, c["wantreg"] and c["mtype"] == sw.NRM_CAUCHY)
    assert a[0] != 1.25


def test_regularize_3d_and_eps_from_ratios(ctx, oracle):
    """3D model with the y pass, Z_weights, both terms with compute_eps and
    compute_eps_log at evaluation 0, then a later evaluation that keeps
    them."""
    nz, nx, ny = 40, 50, 12
    vel = _model(nz, nx, ny, seed=6)
    d = sw.reg_desc(nz, nx, ny, wantreg=True, wantlog=True, derivdx=True, derivdy=True,
                    derivdz=True, log_z_plus=True, tapery=3, model_nrm_type=sw.NRM_HUBER,
                    hinge_nrm_type=sw.NRM_L1, compute_eps=True, compute_eps_log=True,
                    ratio=5.0, ratio_log=20.0)
    rng = np.random.default_rng(8)
    grad = rng.standard_normal(vel.size).astype(F)
    zw = (0.5 + rng.random(vel.size)).astype(F)
    a, b = _both(ctx, oracle, d, (0.0, 0.0, 0.0, 0.0), 0, vel, 7.5, grad, zw=zw)
    _check(a, b, False)
    st = tuple(getattr(a[2], k) for k in ("eps", "eps_log", "mod_thresh", "hin_thresh"))
    assert st[0] > 0 and st[1] > 0
    a, b = _both(ctx, oracle, d, st, 1, vel * F(1.02), 6.0, grad, zw=zw)
    _check(a, b, False)
    assert (a[2].eps, a[2].eps_log) == st[:2]


def test_regularize_without_terms_only_masks(ctx):
    d = sw.reg_desc(20, 30)
    rng = np.random.default_rng(1)
    grad = rng.standard_normal(600).astype(F)
    mask = np.tile(np.array([0, 1, 2], F), 200)
    st = sw.SwRegState(1.0, 1.0, 0.0, 0.0)
    f, g = ctx.fwi_regularize(d, st, 0, _model(20, 30), 2.0, grad, vpmask=mask)
    assert f == 2.0
    np.testing.assert_array_equal(g, grad * mask)


def test_regularize_refuses_eps_from_a_zero_term(ctx):
    """compute_eps with no active derivative: the reference stops with
    'cannot compute eps'; here SW_NUMERIC."""
    d = sw.reg_desc(10, 12, wantreg=True, compute_eps=True)
    st = sw.SwRegState(0.0, 0.0, 0.0, 0.0)
    with pytest.raises(sw.SwaveError) as e:
        ctx.fwi_regularize(d, st, 0, _model(10, 12), 1.0, np.zeros(120, F))
    assert e.value.code == sw.SW_NUMERIC

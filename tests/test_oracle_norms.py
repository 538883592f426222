"""The oracle's data norms (libs/libinv/Norm.f90 through Compute_OF_RES_ADJ,
libs/libwave/Objective_Function_Residual_Adjsource.f90:17-40) against a
loop-by-loop numpy restatement, the threshold reset of a gather, and the
adjoint source as the derivative of the misfit."""
import numpy as np
import pytest

import seismic_gb300 as sw

F = np.float32


def _fct(ntype, rd, thresh):
    """fct_compute with FP32 sums in sample order; returns (f, thresh)."""
    if ntype == sw.NRM_L2:
        s = 0.0
        for v in rd.astype(np.float64):
            s = s + v * v
        return s / 2, thresh
    if ntype == sw.NRM_L1:
        s = F(0)
        for v in rd:
            s = F(s + abs(v))
        return float(s), thresh
    if thresh == 0:
        thresh = F(np.max(np.abs(rd)))
    g = F(thresh)
    s = F(0)
    for r in rd:
        if ntype == sw.NRM_HUBER:
            v = F(abs(r) - g / F(2)) if abs(r) > g else F(r * r / (F(2) * g))
        elif ntype == sw.NRM_CAUCHY:
            q = F(r / g)
            v = F(np.log(F(F(1) + q * q)) / F(2))
        else:
            v = F(np.sqrt(F(g * g + r * r)) - g)
        s = F(s + v)
    return float(s), thresh


def _gdt(ntype, rd, g):
    g = F(g)
    if ntype == sw.NRM_L2:
        return rd
    if ntype == sw.NRM_L1:
        return np.sign(rd).astype(F)
    if ntype == sw.NRM_HUBER:
        return np.clip(rd / g, F(-1), F(1)).astype(F)
    if ntype == sw.NRM_CAUCHY:
        return (rd / (g * g + rd * rd)).astype(F)
    return ((rd / g) / np.sqrt(F(1) + rd * rd / (g * g))).astype(F)


def _gather(ntype, thresh, dobs, dmod, mute):
    f, adj, res = 0.0, np.empty_like(dmod), np.empty_like(dmod)
    for j in range(dobs.shape[0]):
        rd = (mute[j] * (dobs[j] - dmod[j])).astype(F)
        fj, thresh = _fct(ntype, rd, thresh)
        f += fj
        res[j] = rd
        adj[j] = _gdt(ntype, (mute[j] * rd).astype(F), thresh)
    return f, adj, res


def _case(nrec=5, nt=60, seed=0):
    rng = np.random.default_rng(seed)
    dobs = rng.standard_normal((nrec, nt)).astype(F)
    dmod = (0.5 * rng.standard_normal((nrec, nt))).astype(F)
    mute = (rng.random((nrec, nt)) > 0.2).astype(F)
    mute[:, :3] = F(0.5)
    return dobs, dmod, mute


NORMS = [sw.NRM_L1, sw.NRM_L2, sw.NRM_HUBER, sw.NRM_CAUCHY, sw.NRM_HYPERBOLIC]


@pytest.mark.parametrize("ntype", NORMS)
@pytest.mark.parametrize("thresh", [0.0, 0.7])
def test_oracle_norm_matches_restatement(oracle, ntype, thresh):
    dobs, dmod, mute = _case()
    f, adj, res = oracle.data_norm(ntype, thresh, dobs, dmod, mute)
    rf, radj, rres = _gather(ntype, F(thresh), dobs, dmod, mute)
    np.testing.assert_array_equal(res, rres)
    np.testing.assert_array_equal(adj, radj)
    # numpy's float32 log may differ from the C library's by an ulp.
    tol = 1e-6 if ntype == sw.NRM_CAUCHY else 0.0
    assert abs(f - rf) <= tol * abs(rf)


def test_threshold_is_the_first_live_trace_of_the_gather(oracle):
    """With data_threshold = 0 every trace of a gather uses max|r| of its
    first trace whose residual is not all zero; a gather with a different
    first trace gets a different threshold."""
    dobs, dmod, mute = _case(nrec=4)
    mute[0] = 0.0                        # first trace muted: threshold from trace 2
    dobs[1] *= 3.0
    m1 = float(np.max(np.abs(mute[1] * (dobs[1] - dmod[1]))))
    # Trace 0 is all zero with threshold 0: 0/0 in the reference as here.
    f, adj, _ = oracle.data_norm(sw.NRM_HUBER, 0.0, dobs, dmod, mute)
    assert np.isnan(f)
    # From trace 1 on the threshold is m1: compare against an explicit one.
    f1, adj1, _ = oracle.data_norm(sw.NRM_HUBER, 0.0, dobs[1:], dmod[1:], mute[1:])
    f2, adj2, _ = oracle.data_norm(sw.NRM_HUBER, m1, dobs[1:], dmod[1:], mute[1:])
    assert f1 == f2
    np.testing.assert_array_equal(adj1, adj2)
    np.testing.assert_array_equal(adj[1:], adj2)
    # A threshold from each trace's own maximum gives another misfit.
    per_trace = sum(oracle.data_norm(sw.NRM_HUBER, 0.0, dobs[j:j + 1], dmod[j:j + 1],
                                     mute[j:j + 1])[0] for j in range(1, 4))
    assert per_trace != f1


@pytest.mark.parametrize("ntype", [sw.NRM_L2, sw.NRM_HUBER, sw.NRM_CAUCHY, sw.NRM_HYPERBOLIC])
def test_adjoint_source_is_the_misfit_derivative(oracle, ntype):
    """With a fixed threshold, d f / d dmod = -mute * adj (the residual is
    mute*(dobs - dmod)); central differences in FP32 agree to 1e-2."""
    dobs, dmod, mute = _case(nrec=2, nt=40, seed=4)
    g = 0.8
    _, adj, _ = oracle.data_norm(ntype, g, dobs, dmod, mute)
    rng = np.random.default_rng(9)
    for _ in range(6):
        j, t = int(rng.integers(2)), int(rng.integers(3, 40))
        if mute[j, t] == 0:
            continue
        h = 1e-2
        dp, dm = dmod.copy(), dmod.copy()
        dp[j, t] += h
        dm[j, t] -= h
        fp = oracle.data_norm(ntype, g, dobs, dp, mute)[0]
        fm = oracle.data_norm(ntype, g, dobs, dm, mute)[0]
        num = (fp - fm) / (2 * h)
        assert abs(num + adj[j, t]) <= 1e-2 * max(1.0, abs(adj[j, t]))


def test_unknown_norm_is_refused(oracle):
    dobs, dmod, mute = _case(nrec=1, nt=8)
    with pytest.raises(RuntimeError):
        oracle.data_norm(7, 0.0, dobs, dmod, mute)

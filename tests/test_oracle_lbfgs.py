"""The oracle's l_bfgs driver (Inversion.f90:29-189) on an analytic
objective (CPU)."""
import numpy as np


def test_l_bfgs_driver_scaling_and_convergence(oracle):
    """A separable quadratic 0.5 sum a_i (x_i - t_i)^2 (FP64) whose gradient
    the driver receives with the reference's sign (the objective routine
    returns minus the gradient, l_bfgs hands -g to LBFGS): the first entry of
    the 'function' history is max(x0)^2 (the f0 scaling of evaluation 0),
    the scaled misfit falls monotonically over the iterations, the model
    approaches the target, and FREEZE_X keeps it inside [vpmin, vpmax]."""
    rng = np.random.default_rng(4)
    n = 200
    t = rng.uniform(1800.0, 2600.0, n)
    a = rng.uniform(0.5, 2.0, n)
    x0 = np.full(n, 2000.0, np.float32)
    evals = []

    def fctgdt(x, eval_):
        evals.append(eval_)
        r = x.astype(np.float64) - t
        return float(0.5 * np.sum(a * r * r)), (-(a * r)).astype(np.float32)

    x, hist, models = oracle.l_bfgs(fctgdt, x0, niter=8, neval=40, xmin=1500.0, xmax=4500.0)
    assert evals == list(range(len(evals)))
    assert hist[0] == np.float32(2000.0 ** 2)
    assert len(models) == 8 and hist.size == 9
    assert np.all(np.diff(hist.astype(np.float64)) < 0)
    assert np.linalg.norm(x - t) < 0.05 * np.linalg.norm(x0 - t)
    assert x.min() >= 1500.0 and x.max() <= 4500.0


def test_freeze_x_hard_and_soft(oracle):
    """FREEZE_X (lbfgs.f:1-40): soft clips everything; hard clips entries
    whose mask is neither 0 nor 2 and resets the others to the start."""
    x = np.array([1000.0, 5000.0, 3000.0, 9000.0])
    xinit = np.array([1.0, 2.0, 3.0, 4.0])
    mask = np.array([1.0, 0.0, 2.0, 0.5], np.float32)
    soft = oracle.freeze_x(x.copy(), 1500.0, 4500.0, mask, True, xinit)
    np.testing.assert_array_equal(soft, [1500.0, 4500.0, 3000.0, 4500.0])
    hard = oracle.freeze_x(x.copy(), 1500.0, 4500.0, mask, False, xinit)
    np.testing.assert_array_equal(hard, [1500.0, 2.0, 3.0, 4500.0])


def _oc_run(step, n, nparam, t, a, xmin, xmax, lbfgs_type, bound_type, stp1_opt,
            max_calls=400, x0=None):
    """Drives an out-of-core L-BFGS step function (oracle or device) on
    0.5 sum a (x - t)^2 the way L_BFGS.x is driven: every call starts from
    the state the previous one returned."""
    import seismic_gb300 as sw
    m = 5
    d, keep = sw.lbfgs_oc_desc(n, m, nparam, xmin, xmax, lbfgs_type, bound_type, stp1_opt)
    x = np.full(n, 2000.0) if x0 is None else x0.copy()
    w = np.zeros(n * (2 * m + 1) + 2 * m)
    diag = np.zeros(n)
    st = sw.SwLbfgsOcState()
    iflag, myinfo = 0, 0
    xs, fs, trial = [], [], []
    for _ in range(max_calls):
        r = x - t
        f = float(0.5 * np.sum(a * r * r))
        g = a * r
        trial.append(x.copy())
        iflag, myinfo = step(d, x, f, g, w, diag, st, iflag, 0)
        if myinfo == 1:
            xs.append(x.copy())
            fs.append(f)
        if iflag <= 0:
            break
    return x, np.array(fs), xs, trial, iflag


def test_lbfgs_oc_bounds_and_convergence(oracle):
    """LBFGSOC (nlinv_lbfgs.f:31-967) on a two-parameter quadratic whose
    minimum lies inside the bounds but whose first steps leave them: every
    trial model of bound_type 1 and every iterate of bound_type 2 lies
    within its block's [xmin, xmax] (FREEZE_XOC, :1-22), the misfit falls
    and the model converges; LBFGSOLD (lbfgs_type 0) converges too."""
    rng = np.random.default_rng(6)
    n, nparam = 120, 2
    t = np.concatenate([rng.uniform(1600.0, 2400.0, 60), rng.uniform(2.1, 2.5, 60) * 1000])
    a = rng.uniform(0.5, 2.0, n)
    xmin, xmax = np.array([1500.0, 2000.0]), np.array([2500.0, 2600.0])
    lo = np.repeat(xmin, n // nparam)
    hi = np.repeat(xmax, n // nparam)
    for bt in (1, 2):
        x, fs, xs, trial, iflag = _oc_run(oracle.lbfgs_oc_step, n, nparam, t, a, xmin, xmax,
                                          1, bt, 1)
        assert len(xs) >= 5 and np.all(np.diff(fs) <= 0)
        checked = trial[1:] if bt == 1 else xs
        for v in checked:
            assert np.all(v >= lo) and np.all(v <= hi)
        assert np.abs(xs[-1] - t).max() < 5.0
    x, fs, xs, trial, iflag = _oc_run(oracle.lbfgs_oc_step, n, nparam, t, a, None, None, 0, 1, 0)
    assert len(xs) >= 5 and np.abs(xs[-1] - t).max() < 1.0

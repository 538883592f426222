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

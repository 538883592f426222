"""Learned-preconditioned FWI driver (seismic_gb300.precond) on the GPU."""
import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300 import precond as pc

pytestmark = pytest.mark.gpu

KW = dict(nz=40, nx=100, nt=500, nshot=3, f0=5.0, smooth_m=120.0)


def test_zero_network_falls_back_to_plain_lbfgs(ctx):
    """A network whose output is zero never gives a descent direction, so the
    learned method is plain L-BFGS from the start: identical misfit history."""
    sv = pc.make_survey(ctx, seed=4, **KW)
    hp = pc.plain_fwi(ctx, sv, target=0.0, max_evals=8)
    net = sw.CNN(ctx, (2, 8, 1), seed=0)
    try:
        net.set_weights(np.zeros(net.num_weights, np.float32))
        hl = pc.learned_fwi(ctx, sv, net, step_scale=50.0, target=0.0, max_evals=8)
    finally:
        net.close()
    assert hl.learned_steps == 0
    assert hl.misfit == hp.misfit
    assert hp.misfit[-1] < hp.misfit[0]


def test_pairs_training_and_learned_steps(ctx):
    """Pairs from plain runs train the network (loss falls) and the learned
    method accepts only Armijo-checked descent steps (misfit never above the
    start)."""
    x, y, scale = pc.collect_pairs(ctx, seeds=(1000, 1001), max_evals=8, **KW)
    assert x.shape[1] == 2 and x.shape[0] == y.shape[0] >= 4 and scale > 0
    net = sw.CNN(ctx, (2, 16, 16, 1), seed=0)
    try:
        losses = pc.train_cnn(net, x, y, epochs=60, batch=4)
        sv = pc.make_survey(ctx, seed=5, **KW)
        hl = pc.learned_fwi(ctx, sv, net, scale, target=0.0, max_evals=10, c1=0.1)
    finally:
        net.close()
    assert np.mean(losses[-10:]) < losses[0]
    assert hl.evals <= 10 and hl.x is not None
    # every accepted iterate decreased the misfit (trial points may not)
    assert min(hl.misfit) < 1.0


def test_multiscale_study_driver_small(ctx):
    """The multiscale driver (stages of rising frequency, each starting from
    the previous stage's model) and the study around it, on a small copy of
    the benchmark geometry: misfits fall, solves are counted per stage."""
    cfg = dict(pc.CONFIG4, test=(40, 120), train=(30, 90), nshot=3, t=0.5,
               stages=(4.0, 8.0), smooth_m=100.0, nlayers=8, nfaults=2)
    r = pc.run_config4_study(ctx, n_train=2, train_nshot=2, test_seeds=(3,), evals_per_stage=4,
                             train_evals_per_stage=6, epochs=20, channels=(2, 32, 32, 1),
                             cfg=cfg, learned_kw={"max_learned": 2, "c1": 0.1})
    assert r["pairs"] >= 2
    row = r["tests"][0]
    for m in ("plain", "learned"):
        h = row[m]
        assert len(h["stages"]) == 2
        assert h["solves"] == sum(s["solves"] for s in h["stages"]) > 0
        assert h["final_rel_misfit"] < 1.0

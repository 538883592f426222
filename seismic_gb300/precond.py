"""Learned gradient preconditioning for 2D FWI (no reference counterpart).

The plain method is the reference's: compute_fct_gdt for the misfit and
gradient (sw_fwi_fct_gdt) and the device L-BFGS (sw_lbfgs_*, LBFGS of
libs/libinv/lbfgs.f) driven like l_bfgs (Inversion.f90:29-189), which hands
LBFGS the negated compute_fct_gdt gradient.

The learned method maps the raw gradient and the source illumination of the
current model to a search direction with the convolutional network of
sw_cnn_* (tensor-core BF16 convolutions).  The network is trained on
(gradient, illumination) -> L-BFGS step pairs that plain runs produce on
seed-generated models (target: the update from each iterate to the run's
final model).  The learned steps come first; each proposed direction is
used only if it is a descent direction and a short backtracking line search
finds sufficient decrease (Armijo); from the first failure on, plain
L-BFGS takes over.  Both
methods count wave-equation solves: a forward and an adjoint propagation per
shot for every misfit/gradient evaluation.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import SwFwiDesc, make_genpar, synth


@dataclass
class Survey:
    """A small 2D FWI problem: geometry, wavelet, shots and the true model."""
    desc: SwFwiDesc
    wavelet: np.ndarray
    shots: list
    vtrue: np.ndarray
    v0: np.ndarray
    vmin: float
    vmax: float


def make_survey(ctx, seed: int, nz: int = 60, nx: int = 180, d: float = 10.0, nt: int = 900,
                dt: float = 1e-3, nshot: int = 6, f0: float = 8.0, smooth_m: float = 120.0,
                vmin: float = 1500.0, vmax: float = 3500.0, nlayers: int = 8, nfaults: int = 2,
                snapi: int = 2) -> Survey:
    """Seeded layered/faulted model, a smoothed start model and observed data
    modelled with the FWI forward operator (AMOD) on the true model."""
    vtrue = synth.layered_faulted(nz, nx, d, seed=seed, nlayers=nlayers, nfaults=nfaults,
                                  vmin=vmin, vmax=vmax)
    v0 = synth.smooth(vtrue, d, smooth_m)
    g = make_genpar(nz, nx, 1, dz=d, dx=d, dt=dt, nt=nt, ntaper=20, lsinc=7, snapi=snapi,
                    fmax=2.5 * f0)
    desc = SwFwiDesc()
    desc.g = g
    desc.aperture_x, desc.aperture_y = 0.0, 0.0
    desc.illu_pow = 0.0                      # raw gradient (illumination separately)
    desc.smooth_rect1 = desc.smooth_rect2 = desc.smooth_rect3 = 1
    desc.smooth_doz = desc.smooth_dox = desc.smooth_doy = 0
    desc.checkpoint_snaps = 0
    w = synth.ricker(f0, dt, nt)
    xs = np.linspace(0.1, 0.9, nshot) * (nx - 1) * d
    rec = np.zeros((nx // 2, 3), np.float32)
    rec[:, 0] = d
    rec[:, 1] = np.linspace(0.0, (nx - 1) * d, nx // 2)
    shots = [{"sou": np.array([d, sx, 0.0], np.float32), "rec": rec,
              "dobs": np.zeros((rec.shape[0], nt), np.float32)} for sx in xs]
    # Observed data: resid = dobs - dmod with dobs = 0 on the true model.
    _, _, _, res = ctx.fwi_fct_gdt(desc, vtrue, w, shots, want_resid=True)
    for s, r in zip(shots, res):
        s["dobs"] = -r
    return Survey(desc, w, shots, vtrue, v0, vmin, vmax)


@dataclass
class History:
    evals: int = 0
    f0: float = 0.0
    misfit: list = field(default_factory=list)    # relative misfit after each evaluation
    learned_steps: int = 0
    fallback_steps: int = 0
    seconds: float = 0.0
    x: np.ndarray | None = None                     # final model

    def solves(self, nshot: int) -> int:
        return 2 * nshot * self.evals


class _Evaluator:
    def __init__(self, ctx, sv: Survey, hist: History):
        self.ctx, self.sv, self.hist = ctx, sv, hist

    def __call__(self, x: np.ndarray):
        f, g, il = self.ctx.fwi_fct_gdt(self.sv.desc, x.astype(np.float32), self.sv.wavelet,
                                        self.sv.shots)
        self.hist.evals += 1
        if self.hist.f0 == 0.0:
            self.hist.f0 = f
        self.hist.misfit.append(f / self.hist.f0)
        # compute_fct_gdt returns a descent direction; l_bfgs hands LBFGS -g.
        return f, -np.asarray(g, np.float64), np.asarray(il, np.float64)


def plain_fwi(ctx, sv: Survey, target: float = 0.01, max_evals: int = 60, record=None) -> History:
    """L-BFGS (M = 5) until the misfit falls below target * initial misfit
    or max_evals evaluations; when LBFGS stops (IFLAG <= 0, e.g. a failed
    line search) it restarts with empty memory from the current model.
    Trial models of the line search are clipped to [vmin, vmax] (FREEZE_X
    on every trial, bound_type 1): an unclipped trial step can leave the
    velocity range for which the time step is stable.
    record(x, gd, illum) is called at the start model and after every
    completed iteration."""
    from . import LBFGS
    hist = History()
    t0 = time.perf_counter()
    fg = _Evaluator(ctx, sv, hist)
    x = sv.v0.astype(np.float64).ravel().copy()
    f, gd, il = fg(x)
    if record is not None:
        record(x.copy(), gd.copy(), il.copy())
    restarts = 0
    while hist.evals < max_evals and f > target * hist.f0 and restarts < 4:
        lb = LBFGS(ctx, x.size, 5, sv.vmin, sv.vmax, bound_type=1, xinit=x)
        progressed = False
        try:
            while hist.evals < max_evals and f > target * hist.f0:
                iflag, info = lb.step(x, f, gd)
                if iflag <= 0:
                    break
                f, gd, il = fg(x)
                if info == 1:
                    progressed = True
                    if record is not None:
                        record(x.copy(), gd.copy(), il.copy())
        finally:
            lb.close()
        restarts += 0 if progressed else 1
        if not progressed:
            break
    hist.seconds = time.perf_counter() - t0
    hist.x = x.copy()
    return hist


def _features(gd: np.ndarray, il: np.ndarray, shape) -> np.ndarray:
    """Network input: the gradient and the illumination, each scaled to a
    maximum magnitude of 1, as (2, nx, nz)."""
    g = gd.reshape(shape)
    i = il.reshape(shape)
    g = g / max(np.abs(g).max(), 1e-30)
    i = i / max(np.abs(i).max(), 1e-30)
    return np.stack([g, i]).astype(np.float32)


def collect_pairs(ctx, seeds, max_evals: int = 40, **survey_kw):
    """Training pairs from plain runs on seeded models: the features of every
    iterate x_k and, as target, the remaining update x_final - x_k of that
    run scaled to a maximum magnitude of 1.  Also returns the median of the
    updates' maximum magnitudes (the learned method's first trial step)."""
    xs, ys, scales = [], [], []
    for sd in seeds:
        sv = make_survey(ctx, seed=sd, **survey_kw)
        shape = sv.v0.shape
        its = []
        h = plain_fwi(ctx, sv, target=0.0, max_evals=max_evals,
                      record=lambda x, gd, il: its.append((x, gd, il)))
        for x, gd, il in its[:-1]:
            step = h.x - x
            s = np.abs(step).max()
            if s > 0:
                xs.append(_features(gd, il, shape))
                ys.append((step / s).reshape(shape).astype(np.float32))
                scales.append(s)
    return np.stack(xs), np.stack(ys), float(np.median(scales))


def train_cnn(net, x: np.ndarray, y: np.ndarray, epochs: int = 300, batch: int = 8,
              lr: float = 2e-3, seed: int = 0) -> list:
    rng = np.random.default_rng(seed)
    losses = []
    for ep in range(epochs):
        idx = rng.choice(len(x), size=min(batch, len(x)), replace=False)
        losses.append(net.train_step(x[idx], y[idx], lr=lr))
    return losses


def learned_fwi(ctx, sv: Survey, net, step_scale: float, target: float = 0.01,
                max_evals: int = 60, tries: int = 3, max_learned: int = 10,
                c1: float = 1e-4) -> History:
    """Network directions first: each must be a descent direction and pass
    an Armijo backtracking check (trial steps step_scale, /2, /4 in m/s of
    the largest update).  After the first direction that fails, plain
    L-BFGS (with the restarts of plain_fwi) continues from the model reached."""
    from . import LBFGS
    hist = History()
    t0 = time.perf_counter()
    fg = _Evaluator(ctx, sv, hist)
    shape = sv.v0.shape
    x = sv.v0.astype(np.float64).ravel().copy()
    f, gd, il = fg(x)
    while (hist.evals < max_evals and f > target * hist.f0 and
           hist.learned_steps < max_learned):
        d = net.forward(_features(gd, il, shape)).astype(np.float64).ravel()
        slope = float(np.dot(gd, d))
        accepted = False
        if slope < 0 and np.isfinite(slope):
            alpha = step_scale / max(np.abs(d).max(), 1e-30)
            for _ in range(tries):
                xt = np.clip(x + alpha * d, sv.vmin, sv.vmax)
                ft, gt, it = fg(xt)
                if ft <= f + c1 * alpha * slope:
                    x, f, gd, il = xt, ft, gt, it
                    accepted = True
                    break
                alpha *= 0.5
                if hist.evals >= max_evals:
                    break
        if not accepted:
            break
        hist.learned_steps += 1
    # Plain L-BFGS from the model the learned steps reached.
    restarts = 0
    while hist.evals < max_evals and f > target * hist.f0 and restarts < 4:
        lb = LBFGS(ctx, x.size, 5, sv.vmin, sv.vmax, bound_type=1, xinit=x)
        progressed = False
        try:
            while hist.evals < max_evals and f > target * hist.f0:
                iflag, info = lb.step(x, f, gd)
                if iflag <= 0:
                    break
                f, gd, il = fg(x)
                if info == 1:
                    progressed = True
                    hist.fallback_steps += 1
        finally:
            lb.close()
        restarts += 0 if progressed else 1
        if not progressed:
            break
    hist.seconds = time.perf_counter() - t0
    hist.x = x.copy()
    return hist


def model_error(sv: Survey, x: np.ndarray) -> float:
    """L2 model error relative to the start model's."""
    return float(np.linalg.norm(x.ravel() - sv.vtrue.ravel()) /
                 np.linalg.norm(sv.v0.ravel() - sv.vtrue.ravel()))


def run_study(ctx, train_seeds=tuple(range(1000, 1016)), test_seeds=(4, 5, 6), epochs: int = 400,
              channels=(2, 32, 32, 32, 1), max_evals: int = 60, learned_kw=None,
              **survey_kw) -> dict:
    """Trains the network on plain runs over train_seeds, then inverts every
    test model with both methods.  The target misfit is the best one the
    plain method reaches within max_evals evaluations; solves are counted up
    to the first evaluation at or below it."""
    from . import CNN
    t0 = time.perf_counter()
    x, y, scale = collect_pairs(ctx, train_seeds, **survey_kw)
    t_pairs = time.perf_counter() - t0
    net = CNN(ctx, channels, seed=0)
    try:
        t1 = time.perf_counter()
        losses = train_cnn(net, x, y, epochs=epochs)
        t_train = time.perf_counter() - t1
        rows = []
        for sd in test_seeds:
            sv = make_survey(ctx, seed=sd, **survey_kw)
            nshot = len(sv.shots)
            hp = plain_fwi(ctx, sv, target=0.0, max_evals=max_evals)
            tgt = min(hp.misfit)
            ep = 1 + int(np.argmax(np.array(hp.misfit) <= tgt))
            # The learned run goes the full max_evals so that both curves can
            # be read at every misfit level.
            hl = learned_fwi(ctx, sv, net, scale, target=0.0, max_evals=max_evals,
                             **(learned_kw or {}))
            reached = min(hl.misfit) <= tgt
            el = (1 + int(np.argmax(np.array(hl.misfit) <= tgt))) if reached else None

            def evals_to(curve, level):
                c = np.array(curve)
                return 1 + int(np.argmax(c <= level)) if (c <= level).any() else None

            levels = []
            for lv in (0.5, 0.3, 0.2, 0.1, 0.05, 0.02, 0.01):
                a, b = evals_to(hp.misfit, lv), evals_to(hl.misfit, lv)
                levels.append({"rel_misfit": lv, "plain_solves": 2 * nshot * a if a else None,
                               "learned_solves": 2 * nshot * b if b else None,
                               "ratio": (a / b) if (a and b) else None})
            rows.append({
                "solves_to_level": levels,
                "seed": sd, "target_rel_misfit": tgt,
                "plain_solves": 2 * nshot * ep,
                "learned_solves": (2 * nshot * el) if el else None,
                "learned_reached": bool(reached),
                "learned_best_rel_misfit": float(min(hl.misfit)),
                "plain_model_err": model_error(sv, hp.x),
                "learned_model_err": model_error(sv, hl.x),
                "learned_steps": hl.learned_steps, "fallback_steps": hl.fallback_steps,
                "plain_seconds": hp.seconds, "learned_seconds": hl.seconds,
                "plain_curve": [float(m) for m in hp.misfit],
                "learned_curve": [float(m) for m in hl.misfit],
            })
    finally:
        net.close()
    return {"pairs": int(len(x)), "step_scale": scale, "pair_seconds": t_pairs,
            "train_seconds": t_train, "train_loss_first": float(losses[0]),
            "train_loss_last": float(np.mean(losses[-20:])), "tests": rows}


# The learned-preconditioner FWI benchmark: 601 x 1801 test models at 10 m
# from the layered, faulted generator (40 dipping layers, 6 normal faults,
# 3 % correlated noise, 1500-4700 m/s), start model the true model smoothed
# by a Gaussian of 250 m, 80 shots, 4 s records, Ricker stages at 3, 6 and
# 9 Hz; training pairs from plain runs on 301 x 901 models.  dt is 0.9 ms:
# 1 ms exceeds the 2D Courant limit of the 8th-order scheme at 4700 m/s.
CONFIG4 = {"test": (601, 1801), "train": (301, 901), "d": 10.0, "dt": 9e-4, "t": 4.0,
           "nshot": 80, "stages": (3.0, 6.0, 9.0), "smooth_m": 250.0, "vmin": 1500.0,
           "vmax": 4700.0, "nlayers": 40, "nfaults": 6, "snapi": 4}


def _stage_survey(ctx, seed, shape, f0, nshot, cfg, v0=None) -> Survey:
    nz, nx = shape
    sv = make_survey(ctx, seed, nz=nz, nx=nx, d=cfg["d"], nt=int(round(cfg["t"] / cfg["dt"])),
                     dt=cfg["dt"], nshot=nshot, f0=f0, smooth_m=cfg["smooth_m"],
                     vmin=cfg["vmin"], vmax=cfg["vmax"], nlayers=cfg["nlayers"],
                     nfaults=cfg["nfaults"], snapi=cfg["snapi"])
    if v0 is not None:
        sv.v0 = np.asarray(v0, np.float32).reshape(sv.v0.shape)
    return sv


def multiscale_fwi(ctx, seed: int, shape, nshot: int, cfg=CONFIG4, net=None, step_scale=None,
                   evals_per_stage: int = 20, target: float = 0.01, record=None,
                   learned_kw=None) -> dict:
    """One inversion over the frequency stages: plain L-BFGS (net None) or
    learned directions first with the L-BFGS fallback; each stage starts
    from the previous stage's model and stops at `target` times its own
    start misfit or after evals_per_stage evaluations.  The final misfit is
    also stated relative to the last stage's misfit of the original start
    model (one extra evaluation, not counted as solves)."""
    x = None
    stages = []
    solves = 0
    seconds = 0.0
    sv = None
    for f0 in cfg["stages"]:
        sv = _stage_survey(ctx, seed, shape, f0, nshot, cfg, v0=x)
        rec = None if record is None else (lambda xx, gd, il, f0=f0: record(f0, xx, gd, il))
        if net is None:
            h = plain_fwi(ctx, sv, target=target, max_evals=evals_per_stage, record=rec)
        else:
            h = learned_fwi(ctx, sv, net, step_scale, target=target, max_evals=evals_per_stage,
                            **(learned_kw or {}))
        x = h.x
        solves += h.solves(nshot)
        seconds += h.seconds
        stages.append({"f0_hz": f0, "evals": h.evals, "solves": h.solves(nshot),
                       "seconds": h.seconds, "rel_misfit_end": float(h.misfit[-1]),
                       "rel_misfit_best": float(min(h.misfit)),
                       "learned_steps": h.learned_steps, "fallback_steps": h.fallback_steps,
                       "curve": [float(m) for m in h.misfit]})
    # The last stage's misfit of the original start model.
    sv0 = _stage_survey(ctx, seed, shape, cfg["stages"][-1], nshot, cfg)
    f_start, _, _ = _Evaluator(ctx, sv0, History())(sv0.v0.astype(np.float64).ravel())
    f_end, _, _ = _Evaluator(ctx, sv, History())(x)
    return {"solves": solves, "seconds": seconds, "stages": stages,
            "final_rel_misfit": float(f_end / f_start),
            "model_err": model_error(sv0, x), "x": x}


def run_config4_study(ctx, n_train: int = 64, train_nshot: int = 40, test_seeds=(7,),
                      evals_per_stage: int = 20, train_evals_per_stage: int = 12,
                      epochs: int = 600, channels=(2, 32, 32, 32, 1), cfg=CONFIG4,
                      learned_kw=None, log=None) -> dict:
    """Trains the network on pairs from multiscale plain runs over n_train
    seeded models at the training size, then inverts each test model at the
    test size with both methods; solves and wall time per method."""
    from . import CNN
    log = log or (lambda m: None)
    t0 = time.perf_counter()
    xs, ys, scales = [], [], []
    for k, sd in enumerate(range(2000, 2000 + n_train)):
        its = []
        r = multiscale_fwi(ctx, sd, cfg["train"], train_nshot, cfg,
                           evals_per_stage=train_evals_per_stage, target=0.0,
                           record=lambda f0, x, gd, il: its.append((f0, x, gd, il)))
        # Target of each iterate: the remaining update to its stage's end.
        ends = {}
        for f0, x, gd, il in its:
            ends[f0] = x
        shape = (cfg["train"][1], cfg["train"][0])
        for f0, x, gd, il in its:
            step = ends[f0] - x
            s = np.abs(step).max()
            if s > 0:
                xs.append(_features(gd, il, shape))
                ys.append((step / s).reshape(shape).astype(np.float32))
                scales.append(s)
        log(f"training model {k + 1}/{n_train}: {len(xs)} pairs, "
            f"final rel misfit {r['final_rel_misfit']:.3g}")
    t_pairs = time.perf_counter() - t0
    x_tr, y_tr, scale = np.stack(xs), np.stack(ys), float(np.median(scales))
    net = CNN(ctx, channels, seed=0)
    rows = []
    try:
        t1 = time.perf_counter()
        losses = train_cnn(net, x_tr, y_tr, epochs=epochs, batch=8)
        t_train = time.perf_counter() - t1
        log(f"trained: loss {losses[0]:.4g} -> {np.mean(losses[-20:]):.4g} in {t_train:.0f} s")
        for sd in test_seeds:
            hp = multiscale_fwi(ctx, sd, cfg["test"], cfg["nshot"], cfg,
                                evals_per_stage=evals_per_stage)
            log(f"test {sd} plain: {hp['solves']} solves, {hp['seconds']:.0f} s, "
                f"rel misfit {hp['final_rel_misfit']:.3g}")
            hl = multiscale_fwi(ctx, sd, cfg["test"], cfg["nshot"], cfg, net=net,
                                step_scale=scale, evals_per_stage=evals_per_stage,
                                learned_kw=learned_kw)
            log(f"test {sd} learned: {hl['solves']} solves, {hl['seconds']:.0f} s, "
                f"rel misfit {hl['final_rel_misfit']:.3g}")
            for h in (hp, hl):
                h.pop("x")
            rows.append({"seed": sd, "plain": hp, "learned": hl})
    finally:
        net.close()
    return {"train_models": n_train, "train_shape": list(cfg["train"]),
            "train_nshot": train_nshot, "test_shape": list(cfg["test"]),
            "test_nshot": cfg["nshot"], "stages_hz": list(cfg["stages"]), "dt_s": cfg["dt"],
            "record_s": cfg["t"], "pairs": int(len(x_tr)), "step_scale": scale,
            "pair_seconds": t_pairs, "train_seconds": t_train,
            "train_loss_first": float(losses[0]), "train_loss_last": float(np.mean(losses[-20:])),
            "channels": list(channels), "tests": rows}

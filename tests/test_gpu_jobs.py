"""Multi-shot RTM job, FWI objective/gradient and the device L-BFGS against
the oracle, through the C-ABI."""
import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300 import synth
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _survey(nz=50, nx=140, nshot=5, nt_range=(160, 230), seed=3):
    d = 10.0
    dt = 1.5e-3
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, :] * d
    vel = (1800 + 0.9 * z + 60 * rng.standard_normal((nx, nz))).astype(np.float32)
    ntmax = nt_range[1]
    g = sw.make_genpar(nz, nx, 1, dz=d, dx=d, dt=dt, nt=ntmax, ntaper=10, lsinc=7, snapi=4)
    w = synth.ricker(12.0, dt, ntmax)
    shots = []
    for s in range(nshot):
        sx = 200.0 + s * 170.0 + 3.0
        half = rng.uniform(150, 420)
        lo, hi = max(0.0, sx - half), min((nx - 1) * d, sx + half)
        rx = np.arange(np.ceil(lo / d) * d, hi, 2 * d)
        rec = np.zeros((rx.size, 3), np.float32)
        rec[:, 0] = d + 1.0
        rec[:, 1] = rx
        nt = int(rng.integers(*nt_range))
        data = (rng.standard_normal((rx.size, nt)) * 1e-2).astype(np.float32)
        shots.append({"sou": np.array([20.5, sx, 0.0], np.float32), "rec": rec, "data": data})
    return g, vel, w, shots


@pytest.mark.parametrize("max_batch", [1, 2, 16])
def test_rtm_job_matches_oracle(ctx, oracle, max_batch):
    g, vel, w, shots = _survey()
    job = sw.RTMJob(ctx, g, vel, w, shots, aperture_x=100.0)
    job.set_batch(max_batch)
    job.run(0, 2)
    job.run(2, len(shots) - 2)
    im, il, nm = job.result()
    b, pts = job.info()
    job.close()
    rim, ril, rnm = oracle.rtm_job(g, vel, w, shots, aperture_x=100.0)
    assert np.abs(rim).max() > 0
    assert pts > 0 and 1 <= b <= max_batch
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)
    assert rel_l2(nm, rnm) < 1e-6


@pytest.mark.parametrize("kernel", [0, 1, 2, 3, 4])
def test_rtm_job_every_step_kernel(oracle, kernel):
    """The batched RTM (forward with snapshots, backward with injection and
    imaging) is bit-exact with every 2D step kernel: point tiles, streaming,
    TMA tiles (2 CTAs per SM) and the warp-specialised TMA tiles."""
    g, vel, w, shots = _survey(nshot=4, seed=5)
    c = sw.Context(0)
    try:
        c.set_tuning(step_kernel=kernel)
        job = sw.RTMJob(c, g, vel, w, shots, aperture_x=100.0)
        job.set_batch(4)
        job.run()
        im, il, _ = job.result()
        job.close()
    finally:
        c.close()
    rim, ril, _ = oracle.rtm_job(g, vel, w, shots, aperture_x=100.0)
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


def _fwi_case():
    g, vel, w, shots = _survey(nshot=3, nt_range=(200, 201), seed=7)
    rng = np.random.default_rng(11)
    for s in shots:
        s["dobs"] = s.pop("data")
        s["mute"] = (rng.random(s["dobs"].shape) > 0.1).astype(np.float32)
    g.nt = shots[0]["dobs"].shape[1]    # FWI shots share one record length
    d = sw.SwFwiDesc()
    d.g = g
    d.aperture_x, d.aperture_y, d.illu_pow = 50.0, 0.0, 1.0
    d.smooth_rect1, d.smooth_rect2, d.smooth_rect3 = 3, 5, 1
    d.smooth_doz, d.smooth_dox, d.smooth_doy = 1, 1, 0
    mask = np.ones(vel.size, np.float32)
    mask[:5] = 0
    return d, vel, w, shots, mask


def test_fwi_fct_gdt_matches_oracle(ctx, oracle):
    d, vel, w, shots, mask = _fwi_case()
    f, grad, illum = ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    rf, rgrad, rillum = oracle.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    assert rf > 0
    assert f == rf                       # FP64 misfit summed in the same order
    assert rel_l2(grad, rgrad) < 1e-6    # FP32 gradient; one FP64 norm differs in order
    assert rel_l2(illum, rillum) < 1e-6


@pytest.mark.parametrize("ntype", [sw.NRM_L1, sw.NRM_HUBER, sw.NRM_CAUCHY, sw.NRM_HYPERBOLIC])
@pytest.mark.parametrize("thresh", [0.0, 0.01])
def test_fwi_data_norms_match_oracle(ctx, oracle, ntype, thresh):
    """The L1, Huber, Cauchy and hyperbolic misfits and adjoint sources
    (Norm.f90) with data_threshold 0 (each gather's threshold from its first
    live trace) and a fixed one: residuals bit-exact, misfit bit-exact except
    Cauchy, whose FP32 log is CUDA's logf against the C library's (1e-6)."""
    d, vel, w, shots, mask = _fwi_case()
    d.dat_nrm_type, d.dat_thresh = ntype, thresh
    f, grad, illum, gres = ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask, want_resid=True)
    for s in shots:
        s["resid"] = np.zeros(s["dobs"].shape, np.float32)
    rf, rgrad, rillum = oracle.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    for s, r in zip(shots, gres):
        np.testing.assert_array_equal(r, s["resid"])
    assert rf > 0
    if ntype == sw.NRM_CAUCHY:
        assert abs(f - rf) <= 1e-6 * rf
    else:
        assert f == rf
    assert rel_l2(grad, rgrad) < 1e-6
    assert rel_l2(illum, rillum) < 1e-6


def test_fwi_bad_norm_is_refused(ctx):
    d, vel, w, shots, mask = _fwi_case()
    d.dat_nrm_type = 5
    with pytest.raises(sw.SwaveError) as e:
        ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    assert e.value.code == sw.SW_BAD_PARAM


@pytest.mark.parametrize("K", [2, 3, 7])
def test_fwi_checkpointed_equals_store_all(ctx, K):
    """Checkpointed snapshots (state every K snapshots, K + 2 recomputed at a
    time in the backward pass) give the store-all misfit and gradient bit for
    bit: the recomputed forward steps repeat the same operations."""
    d, vel, w, shots, mask = _fwi_case()
    d.checkpoint_snaps = 0
    f0, g0, il0 = ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    ctx.reset_stats()
    d.checkpoint_snaps = K
    f1, g1, il1 = ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    pts_ck = ctx.stats()["points_updated"]
    assert f1 == f0
    np.testing.assert_array_equal(g1, g0)
    np.testing.assert_array_equal(il1, il0)
    # One extra forward propagation; each segment recomputes K + 2 snapshot
    # intervals, so the recomputation is about (K + 2) / K forward runs.
    ctx.reset_stats()
    d.checkpoint_snaps = 0
    ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    pts_all = ctx.stats()["points_updated"]
    assert 1.4 * pts_all < pts_ck <= (1.0 + (K + 2) / (2.0 * K) + 0.02) * pts_all


def _binomial_advances(l, s):
    """t(l, c) with c = s + 1 checkpoints (Griewank 1992): the fewest
    segment advances that reverse l segments."""
    from math import comb
    if l <= 1:
        return 0
    c = s + 1
    r = 0
    while comb(c + r, c) < l:
        r += 1
    return r * l - (comb(c + 1 + r - 1, c + 1) if r >= 1 else 0)


@pytest.mark.parametrize("K,slots", [(2, 1), (2, 2), (2, 3), (3, 1), (2, 100)])
def test_fwi_revolve_equals_store_all(ctx, K, slots):
    """The binomial (revolve) schedule over checkpoint segments gives the
    store-all misfit and gradient bit for bit, with the number of segment
    advances the binomial formula gives for slots + 1 checkpoints (the zero
    initial state is the first), and no more forward steps than the
    uniform scheme needs when slots cover every segment boundary."""
    d, vel, w, shots, mask = _fwi_case()
    d.checkpoint_snaps = 0
    d.revolve_slots = 0
    f0, g0, il0 = ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    d.checkpoint_snaps = K
    d.revolve_slots = slots
    ctx.reset_stats()
    f1, g1, il1 = ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    st = ctx.stats()
    assert f1 == f0
    np.testing.assert_array_equal(g1, g0)
    np.testing.assert_array_equal(il1, il0)
    ntsnap = d.g.nt // d.g.snapi
    nseg = (ntsnap + K - 1) // K
    s_eff = min(slots, nseg - 1)
    assert st["ckpt_advances"] == len(shots) * _binomial_advances(nseg, s_eff)
    d.revolve_slots = 0
    ctx.reset_stats()
    ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    uni = ctx.stats()
    assert uni["ckpt_advances"] == len(shots) * (nseg - 1)
    assert st["steps_backward"] == uni["steps_backward"]
    if s_eff == nseg - 1:
        assert st["steps_forward"] <= uni["steps_forward"]
    else:
        assert st["steps_forward"] > uni["steps_forward"]
    d.checkpoint_snaps = 0


def test_lbfgs_device_matches_oracle(ctx, oracle):
    """A few LBFGS iterations on a bound-constrained quadratic."""
    n = 5000
    rng = np.random.default_rng(3)
    diag = rng.uniform(0.5, 4.0, n)
    xs = rng.uniform(1800, 4000, n)

    def fg(x):
        r = x - xs
        return 0.5 * float(np.sum(diag * r * r)), diag * r

    x0 = np.full(n, 3000.0)
    runs = []
    for impl in ("gpu", "cpu"):
        x = x0.copy()
        opt = (sw.LBFGS(ctx, n, 5, 1500.0, 4500.0, xinit=x0) if impl == "gpu"
               else oracle.LBFGS(n, 5, 1500.0, 4500.0, xinit=x0))
        fs = []
        for _ in range(40):
            f, g = fg(x)
            fs.append(f)
            iflag, info = opt.step(x, f, g)
            if iflag <= 0:
                break
        runs.append((x.copy(), fs, opt.diag()))
        if impl == "gpu":
            opt.close()
    (xg, fg_, dg), (xc, fc, dc) = runs
    assert fg_[-1] < 1e-3 * fg_[0]
    assert len(fg_) == len(fc)
    # Same trajectory up to FP64 reduction order (dot products are tree sums
    # on the device, sequential on the CPU).
    np.testing.assert_allclose(fg_, fc, rtol=1e-6, atol=1e-12 * fc[0])
    np.testing.assert_allclose(xg, xc, rtol=1e-9)


def _window(g, sou, rec, apx):
    """extract_coord_source_receiver_patch in float32 (ExtractPadModel.f90:19-85)."""
    f = np.float32
    sx = f(sou[1])
    gx1, gxn = f(rec[:, 1].min()), f(rec[:, 1].max())
    minx, maxx = min(sx, gx1), max(sx, gxn)
    mx1, mxn = (gx1 + sx) / f(2), (gxn + sx) / f(2)
    cx = mx1 + abs(mxn - mx1) / f(2)
    oxw = min(minx, cx - f(apx) / f(2))
    endx = max(maxx, cx + f(apx) / f(2))
    nxw = int(np.round((endx - oxw) / f(g.dx))) + 1
    return float(oxw), nxw


def test_batched_modeling_matches_oracle(ctx, oracle):
    g, vel, w, shots = _survey(nshot=4, seed=9)
    apx = 0.0
    job = sw.RTMJob(ctx, g, vel, w, [{"sou": s["sou"], "rec": s["rec"], "nt": s["data"].shape[1]}
                                     for s in shots], aperture_x=apx)
    job.set_batch(3)
    out = job.model()
    job.close()
    for s, d in zip(shots, out):
        oxw, nxw = _window(g, s["sou"], s["rec"], apx)
        i0 = int(round(oxw / g.dx))
        gw = sw.make_genpar(g.nz, nxw, 1, dz=g.dz, dx=g.dx, ox=oxw, dt=g.dt, nt=d.shape[1],
                            ntaper=g.ntaper, lsinc=g.lsinc, snapi=g.snapi)
        ref = oracle.modeling(gw, vel[i0:i0 + nxw], s["sou"], w[: d.shape[1]], s["rec"])
        assert np.abs(ref).max() > 0
        np.testing.assert_array_equal(d, ref)


def test_autotuner_on_device(oracle, tmp_path):
    """tune_rtm times every candidate on a truncated copy of the batch, caches
    the winner per device / grid bucket / batch size and applies it; the
    tuned job still matches the oracle bit for bit."""
    from seismic_gb300 import autotune
    g, vel, w, shots = _survey(nshot=3, seed=9)
    c = sw.Context(0)
    try:
        path = str(tmp_path / "tuning.json")
        entry = autotune.tune_rtm(c, g, vel, w, shots, steps=32, cache_path=path)
        assert entry["tuning"] in autotune.candidates(True)
        assert entry["tried"] == len(autotune.candidates(True))
        again = autotune.tune_rtm(c, g, vel, w, shots, steps=32, cache_path=path)
        assert again["tuning"] == entry["tuning"]       # served from the cache
        assert c.tuning()["step_kernel"] == entry["tuning"]["step_kernel"]
        job = sw.RTMJob(c, g, vel, w, shots)
        job.set_batch(3)
        job.run()
        im, il, _ = job.result()
        job.close()
    finally:
        c.close()
    rim, ril, _ = oracle.rtm_job(g, vel, w, shots)
    np.testing.assert_array_equal(im, rim)


def test_autotuner_chooses_shots_per_launch(oracle, tmp_path):
    """tune_rtm(batch="auto") times each batch size on the same shot sample,
    then the launch shape at the chosen size; the job run with both stays
    bit-exact with the oracle."""
    from seismic_gb300 import autotune
    g, vel, w, shots = _survey(nshot=5, seed=13)
    c = sw.Context(0)
    try:
        path = str(tmp_path / "tuning.json")
        entry = autotune.tune_rtm(c, g, vel, w, shots, steps=24, batch="auto", cache_path=path)
        assert entry["batch"] in autotune.batch_candidates(len(shots))
        cached = autotune.load_cache(path)
        times = next(v for k, v in cached.items() if k.endswith("|batch"))["seconds"]
        assert set(times) == {str(b) for b in autotune.batch_candidates(len(shots))}
        job = sw.RTMJob(c, g, vel, w, shots)
        job.set_batch(entry["batch"])
        job.run()
        im, il, _ = job.result()
        job.close()
    finally:
        c.close()
    rim, ril, _ = oracle.rtm_job(g, vel, w, shots)
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


def test_rtm_job_admit_matches_the_batch_run(ctx):
    """sw_rtm_job_admit reports the batch that the next run takes: capped by
    max_shots and by the end of the survey, and SW_OOM_ADMISSION when one
    shot exceeds the memory budget."""
    g, vel, w, shots = _survey(nshot=5, seed=4)
    job = sw.RTMJob(ctx, g, vel, w, shots)
    try:
        job.set_batch(2)
        assert job.admit(0) == 2 and job.admit(4) == 1
        job.run(0, 2)
        assert job.info()[0] == 2
        job.set_batch(64)
        assert job.admit(0) == 5 and job.admit(0, modeling=True) == 5
        job.set_batch(64, 1e-9)
        with pytest.raises(sw.SwaveError) as e:
            job.admit(0)
        assert e.value.code == sw.SW_OOM_ADMISSION
    finally:
        job.close()


def test_tune_survey_on_device(oracle, tmp_path):
    """tune_survey caps the batch candidates by the admission at full record
    length, picks the shots per launch and then the launch shape; the survey
    migrated with its choice stays bit-exact with the oracle."""
    from seismic_gb300 import autotune
    g, vel, w, shots = _survey(nshot=5, seed=21)
    full = [dict(s, nt=s["data"].shape[1]) for s in shots]
    c = sw.Context(0)
    try:
        entry = autotune.tune_survey(c, g, vel, w, full, steps=24,
                                     cache_path=str(tmp_path / "tuning.json"))
        assert entry["admit_cap"] == 5
        assert entry["batch"] in (1, 2, 4, 5)
        assert entry["tuning"] in autotune.candidates(True)
        job = sw.RTMJob(c, g, vel, w, shots)
        job.set_batch(entry["batch"])
        job.run()
        im, il, _ = job.result()
        job.close()
    finally:
        c.close()
    rim, ril, _ = oracle.rtm_job(g, vel, w, shots)
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


def test_fwi_gradient_fd_check_on_device(oracle):
    """The device's raw FWI gradient against centred finite differences of
    the device's misfit along the 8 seeded smooth directions of the oracle's
    check (rigid boundary, illu_pow 0, no smoothing, snapi 1, 6 Hz; see
    tests/test_oracle_pins.py:fd_gradient_check), to the same bound, and the
    device's raw gradient against the oracle's."""
    from tests.test_oracle_pins import check_fd, fd_gradient_check
    c = sw.Context(0)
    try:
        c.set_boundary(1)

        def fct_gdt(desc, vel, w, shots):
            want = all("resid" in s for s in shots)
            out = c.fwi_fct_gdt(desc, vel, w, shots, want_resid=want)
            if want:
                for s, r in zip(shots, out[3]):
                    s["resid"][...] = r
            return out[0], out[1]

        an, fd = fd_gradient_check(fct_gdt)
    finally:
        c.close()
    check_fd(an, fd)
    oracle.set_rigid(True)
    try:
        ran, rfd = fd_gradient_check(
            lambda desc, vel, w, shots: oracle.fwi_fct_gdt(desc, vel, w, shots)[:2])
    finally:
        oracle.set_rigid(False)
    np.testing.assert_array_equal(fd, rfd)       # FP64 misfits summed in the same order
    assert rel_l2(an, ran) < 1e-6


def test_fwi_non_finite_data_is_reported(ctx):
    """A NaN in the observed data reaches the FP64 misfit: sw_fwi_fct_gdt
    returns SW_NUMERIC instead of a NaN misfit."""
    d, vel, w, shots, mask = _fwi_case()
    shots[1]["dobs"] = shots[1]["dobs"].copy()
    shots[1]["dobs"][3, 17] = np.nan
    with pytest.raises(sw.SwaveError) as e:
        ctx.fwi_fct_gdt(d, vel, w, shots, vpmask=mask)
    assert e.value.code == sw.SW_NUMERIC


def test_rtm_job_3d_window_bitexact(ctx, oracle):
    """The multi-shot RTM job in 3D on a 60 x 90 x 80 model (10 m; compute
    windows of about 0.6 million points): two shots of different source
    position and receiver patch migrated in one batch by the pipelined 3D
    kernel, stacked image and
    illumination bit-exact with the oracle's RTM_to_memory per window and
    mod_copy_image (to_disk_to_memory_RTM.f90:358-492,
    ExtractPadModel.f90:662-697)."""
    from tests.cases import model3d
    nz, nx, ny, d, dt, nt = 60, 90, 80, 10.0, 1.5e-3, 200
    g = sw.make_genpar(nz, nx, ny, dz=d, dx=d, dy=d, dt=dt, nt=nt, ntaper=10, lsinc=7, snapi=4,
                       twoD=False, fmax=30.0)
    vel = model3d(nz, nx, ny, d, seed=4)
    w = synth.ricker(12.0, dt, nt)
    shots = []
    for (sx, sy, half) in ((300.0 + 2.0, 350.0 - 1.0, 250.0), (560.0, 420.0 + 3.0, 200.0)):
        gx, gy = np.meshgrid(np.arange(sx - half, sx + half, 30.0),
                             np.arange(sy - half, sy + half, 30.0), indexing="ij")
        keep = (gx >= 0) & (gx <= (nx - 1) * d) & (gy >= 0) & (gy <= (ny - 1) * d)
        rec = np.zeros((int(keep.sum()), 3), np.float32)
        rec[:, 0], rec[:, 1], rec[:, 2] = d + 1.0, gx[keep], gy[keep]
        shots.append({"sou": np.array([25.0, sx, sy], np.float32), "rec": rec, "nt": nt})
    mj = sw.RTMJob(ctx, g, vel, w, shots, aperture_x=100.0, aperture_y=100.0)
    mj.set_batch(2)
    data = mj.model()
    mj.close()
    job_shots = [{"sou": s["sou"], "rec": s["rec"], "data": dd} for s, dd in zip(shots, data)]
    job = sw.RTMJob(ctx, g, vel, w, job_shots, aperture_x=100.0, aperture_y=100.0)
    job.set_batch(2)
    job.run()
    im, il, _ = job.result()
    b, pts = job.info()
    job.close()
    rim, ril, _ = oracle.rtm_job(g, vel, w, job_shots, aperture_x=100.0, aperture_y=100.0)
    assert b == 2 and pts > 200_000_000
    assert np.abs(rim).max() > 0
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


def _oc_misfit(x, t, a):
    r = x - t
    return float(0.5 * np.sum(a * r * r))


@pytest.mark.parametrize("lbfgs_type,bound_type", [(1, 1), (1, 2), (0, 1)])
def test_lbfgs_oc_device_matches_oracle(ctx, oracle, lbfgs_type, bound_type):
    """The out-of-core L-BFGS (LBFGSOC / LBFGSOLD, nlinv_lbfgs.f) on the
    device against the oracle, each call starting from the state the
    previous call returned (as L_BFGS.x does through its files): trial
    models and iterates equal to 1e-9 relative (FP64 dot products summed in
    another order) down to rounding level, and both runs converged."""
    from tests.test_oracle_lbfgs import _oc_run
    rng = np.random.default_rng(12)
    n, nparam = 2000, 2
    t = np.concatenate([rng.uniform(1600.0, 2400.0, n // 2), rng.uniform(2100.0, 2500.0, n // 2)])
    a = rng.uniform(0.5, 2.0, n)
    xmin, xmax = np.array([1500.0, 2000.0]), np.array([2500.0, 2600.0])

    def dev(d, x, f, g, w, diag, st, iflag, myinfo):
        return ctx.lbfgs_oc_step(d, x, f, g, w, diag, st, iflag, myinfo)

    rx, rfs, rxs, rtrial, rfl = _oc_run(oracle.lbfgs_oc_step, n, nparam, t, a, xmin, xmax,
                                        lbfgs_type, bound_type, 1, max_calls=60)
    x, fs, xs, trial, fl = _oc_run(dev, n, nparam, t, a, xmin, xmax, lbfgs_type, bound_type, 1,
                                   max_calls=60)
    # Both runs drive the misfit from 1e8 to rounding level (1e-20 and
    # below, where the last iterations' line searches act on differences
    # of a few ulps); there the number of calls depends on summation
    # order, so the trajectories are compared while the misfit is above
    # 1e-12 of its start, and both must end converged.
    f0 = _oc_misfit(rtrial[0], t, a)
    keep = [i for i, v in enumerate(rtrial) if _oc_misfit(v, t, a) > 1e-12 * f0]
    assert len(keep) >= 5 and len(trial) > keep[-1] and fl == rfl == 0
    for i in keep:
        assert np.abs(trial[i] - rtrial[i]).max() <= 1e-9 * np.abs(rtrial[i]).max()
    nk = sum(1 for v in rfs if v > 1e-12 * f0)
    assert nk >= 5 and rel_l2(fs[:nk], rfs[:nk]) < 1e-9
    assert _oc_misfit(x, t, a) < 1e-12 * f0 and _oc_misfit(rx, t, a) < 1e-12 * f0

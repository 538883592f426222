"""Parity at the benchmark sizes, through the C-ABI.

* The batched RTM survey (751 x 2301 at 4 m, dt 0.375 ms): two shots of
  different aperture and record length (502-column and 1492-column windows,
  8796 and 10569 samples: whole records) modelled and migrated
  together in one batch of the persistent multi-shot kernels, against the
  oracle's modelling and its stacked RTM (RTM_to_memory + mod_copy_image,
  progs/rtm/to_disk_to_memory_RTM.f90:358-492,
  ExtractPadModel.f90:662-697).
* The Born grid (1201 x 3401 at 6.25 m, dt 0.5 ms): one Born shot and its
  LSRTM adjoint on the full grid (records cut to 1000 samples) against the
  oracle (BORN_to_memory, to_disk_to_memory_BORN.f90:123-220;
  LSRTM_to_memory, to_disk_to_memory_RTM.f90:494-580), and the
  rigid-boundary dot-product test of the pair on that grid.
"""
import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300 import synth
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _config2_window_genpar(shot):
    c = synth.CONFIG2
    i0, nxw = synth.config2_window(shot)
    gw = sw.make_genpar(c["nz"], nxw, 1, dz=c["d"], dx=c["d"], ox=i0 * c["d"], dt=c["dt"],
                        nt=shot["nt"], ntaper=c["ntaper"], lsinc=7, snapi=c["snapi"])
    return gw, i0, nxw


def test_config2_two_shots_batched_bitexact(ctx, oracle):
    g, vel, w, shots = synth.config2()
    pick = [shots[0], shots[111]]
    assert synth.config2_window(pick[0])[1] != synth.config2_window(pick[1])[1]
    assert pick[0]["nt"] != pick[1]["nt"]
    # Batched forward modelling of both shots in the same launches.
    mj = sw.RTMJob(ctx, g, vel, w, [{"sou": s["sou"], "rec": s["rec"], "nt": s["nt"]}
                                    for s in pick])
    mj.set_batch(2)
    data = mj.model()
    mj.close()
    for s, d in zip(pick, data):
        gw, i0, nxw = _config2_window_genpar(s)
        ref = oracle.modeling(gw, vel[i0:i0 + nxw], s["sou"], w[: s["nt"]], s["rec"])
        assert np.abs(ref).max() > 0
        np.testing.assert_array_equal(d, ref)
    # Batched RTM of both shots with those data, stacked into the full grid.
    job_shots = [{"sou": s["sou"], "rec": s["rec"], "data": d} for s, d in zip(pick, data)]
    job = sw.RTMJob(ctx, g, vel, w, job_shots)
    job.set_batch(2)
    job.run()
    im, il, nm = job.result()
    b, _ = job.info()
    job.close()
    assert b == 2
    rim, ril, rnm = oracle.rtm_job(g, vel, w, job_shots)
    assert np.abs(rim).max() > 0
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)
    # The normalisation's mean square is one FP64 sum in another order.
    assert rel_l2(nm, rnm) < 1e-6


@pytest.fixture(scope="module")
def config3_case():
    c = synth.config3(nt=1000)
    sou = c["shots"][len(c["shots"]) // 2]
    wb = sw.born_wavelet(c["wavelet"], c["g"].dt)
    return c, sou, wb


def test_config3_born_and_lsrtm_full_grid_bitexact(ctx, oracle, config3_case):
    c, sou, wb = config3_case
    g, vel, ref, rec = c["g"], c["vel"], c["ref"], c["rec"]
    d = ctx.born(g, vel, ref, sou, wb, rec)
    rd = oracle.born(g, vel, ref, sou, wb, rec)
    assert np.abs(rd).max() > 0
    np.testing.assert_array_equal(d, rd)
    im, il = ctx.lsrtm(g, vel, sou, wb, rec, d)
    rim, ril = oracle.lsrtm(g, vel, sou, wb, rec, rd)
    assert np.abs(rim).max() > 0
    np.testing.assert_array_equal(im, rim)
    np.testing.assert_array_equal(il, ril)


def test_config3_dot_test_rigid_full_grid(config3_case):
    """<L m, d> = <m, L^T d> for the Born / LSRTM pair with the rigid
    boundary (exact adjoints), m and d ~ N(0, 1) (seed 33), FP32 operators on
    the GPU, FP64 inner products.  White m and d make <L m, d> small against
    |L m| |d| (by about the square root of the 1.7 million data samples), so
    FP32 rounding of the operators (relative 1e-8) shows up amplified in the
    relative gap: measured 2.5e-5 on this grid, against the 1e-5 that the
    toy-size test meets (test_born_lsrtm_dot_test_rigid) and the oracle's FP64
    pair meets to 1e-12.  The gap against |L m| |d|, free of that
    cancellation, is at FP32 rounding level."""
    c, sou, wb = config3_case
    g, vel, rec = c["g"], c["vel"], c["rec"]
    rng = np.random.default_rng(33)
    m = rng.standard_normal(vel.shape).astype(np.float32)
    d = rng.standard_normal((rec.shape[0], g.nt)).astype(np.float32)
    cx = sw.Context(0)
    try:
        cx.set_boundary(1)
        lm = cx.born(g, vel, m, sou, wb, rec)
        ltd, _ = cx.lsrtm(g, vel, sou, wb, rec, d)
    finally:
        cx.close()
    a = float(np.sum(lm.astype(np.float64) * d))
    b = float(np.sum(m.ravel().astype(np.float64) * ltd.ravel()))
    gap = abs(a - b) / max(abs(a), abs(b))
    scale = float(np.linalg.norm(lm.astype(np.float64)) * np.linalg.norm(d.astype(np.float64)))
    print(f"config-3 grid dot test: <Lm,d>={a:.9e} <m,L^T d>={b:.9e} gap={gap:.2e} "
          f"gap/(|Lm||d|)={abs(a - b) / scale:.2e}")
    assert gap < 1e-4
    assert abs(a - b) / scale < 1e-7

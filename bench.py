#!/usr/bin/env python3
"""Benchmark: batched 2D shot RTM (zero-lag imaging, illumination-normalised
image) on a 751 x 2301 grid at 4 m, dt 0.375 ms, 3-4 s records, 3-6 km
per-shot apertures, 20 Hz Ricker, shots every 37.5 m.

One step = the RTM (forward propagation with snapshots + backward
propagation with imaging) of one batch of shots that advance together in
the same kernel launches.  Metric: FD point updates per second over the
compute domain (interior + 2*ntaper per axis), whole job, and the fused step
kernel's fraction of the measured HBM bandwidth.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N>1) every rank migrates its own shots (weak scaling) and the
stacked images are summed with one all-reduce at the end of the timed region.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NZ, NX, D = 751, 2301, 4.0
DT = 3.75e-4          # the stated 0.4 ms violates the scheme's Courant limit
SNAPI = 4
NTAPER = 20
F0 = 20.0
NSHOT_SURVEY = 240
SPACING = 37.5
BYTES_PER_POINT = 24  # u2, u1, u0, u_1, vel read + u3 written, FP32


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# Workload
# ---------------------------------------------------------------------------
def make_workload(nt_cap: int | None = None):
    """The 240-shot survey (seismic_gb300.synth.config2): full-model genpar,
    vel (nx, nz) = Fortran (nz, nx), wavelet, shots."""
    from seismic_gb300 import synth
    return synth.config2(nt_cap)


def window_of(shot):
    """Columns [i0, i0+nxw) of the shot window (aperture 0: source + spread)."""
    from seismic_gb300 import synth
    return synth.config2_window(shot)


def shot_points(shot, forward_and_back=True):
    i0, nxw = window_of(shot)
    n1 = NZ + 2 * NTAPER
    n2 = nxw + 2 * NTAPER
    return n1 * n2 * shot["nt"] * (2 if forward_and_back else 1)


# ---------------------------------------------------------------------------
# Clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (a restatement of the reference CPU path)
# ---------------------------------------------------------------------------
def cpu_sample(g, vel, w, shot, nsteps: int) -> dict:
    """Times the oracle's RTM of one shot (its whole record when nsteps is 0,
    else truncated to nsteps samples) on random data (the reference arm:
    the time does not depend on the data values)."""
    import seismic_gb300 as sw
    from oracle import bind as oracle
    nsteps = nsteps or shot["nt"]
    i0, nxw = window_of(shot)
    gw = sw.make_genpar(NZ, nxw, 1, dz=D, dx=D, ox=i0 * D, dt=DT, nt=nsteps, ntaper=NTAPER,
                        lsinc=7, snapi=SNAPI)
    rng = np.random.default_rng(0)
    data = rng.standard_normal((shot["rec"].shape[0], nsteps)).astype(np.float32) * 1e-3
    oracle.load()
    t0 = time.perf_counter()
    oracle.rtm(gw, vel[i0:i0 + nxw], shot["sou"], w[:nsteps], shot["rec"], data)
    dt = time.perf_counter() - t0
    pts = (NZ + 2 * NTAPER) * (nxw + 2 * NTAPER) * nsteps * 2
    return {"seconds": dt, "points": pts}


def cpu_parity_sample(ctx, g, vel, w, shots) -> tuple[dict, dict]:
    """The CPU baseline and the parity check of the benchmarked workload:
    the oracle's stacked RTM (RTM_to_memory per shot window + mod_copy_image)
    of `shots` with the very data the GPU migrated, timed on the host cores,
    against the same shots migrated together in one batch on the GPU; and
    the oracle's modelling of the first shot against the GPU-modelled data."""
    import seismic_gb300 as sw
    from oracle import bind as oracle
    oracle.load()
    job = sw.RTMJob(ctx, g, vel, w, shots)
    job.set_batch(len(shots))
    job.run()
    im, il = job.result(normalised=False)
    job.close()
    t0 = time.perf_counter()
    rim, ril, _ = oracle.rtm_job(g, vel, w, shots)
    secs = time.perf_counter() - t0
    pts = sum(shot_points(dict(s, nt=s["data"].shape[1])) for s in shots)
    s0 = shots[0]
    i0, nxw = window_of(s0)
    nt0 = s0["data"].shape[1]
    gw = sw.make_genpar(NZ, nxw, 1, dz=D, dx=D, ox=i0 * D, dt=DT, nt=nt0, ntaper=NTAPER,
                        lsinc=7, snapi=SNAPI)
    gw.surf_type, gw.shot_type, gw.rec_type = g.surf_type, g.shot_type, g.rec_type
    rdata = oracle.modeling(gw, vel[i0:i0 + nxw], s0["sou"], w[:nt0], s0["rec"])

    def rel(a, b):
        den = float(np.linalg.norm(b.astype(np.float64)))
        return float(np.linalg.norm((a.astype(np.float64) - b)) / (den or 1.0))

    parity = {"shots": [float(s["sou"][1]) for s in shots],
              "windows": [window_of(s)[1] for s in shots],
              "records": [int(s["data"].shape[1]) for s in shots],
              "batch": len(shots),
              "image_rel_l2": rel(im, rim), "illum_rel_l2": rel(il, ril),
              "data_rel_l2": rel(s0["data"], rdata),
              "bitexact": bool(np.array_equal(im, rim) and np.array_equal(il, ril)
                               and np.array_equal(s0["data"], rdata))}
    return {"seconds": secs, "points": pts}, parity


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    g, vel, w, shots = make_workload()
    nsteps = args.cpu_steps
    res = []
    for k in range(args.warmup + args.steps):
        r = cpu_sample(g, vel, w, shots[k % len(shots)], nsteps)
        if k >= args.warmup:
            res.append(r)
    nsteps = nsteps or "all"
    secs = sum(r["seconds"] for r in res)
    pts = sum(r["points"] for r in res)
    v = pts / secs / 1e9
    cores = cpu_threads()
    sample = (f"RTM (forward + backward, {nsteps} of the 8000-10667 time samples) of one "
              f"{NZ}x(window) shot per step, {args.steps} steps, {secs:.1f} s")
    line = {
        "impl": "reference", "metric": "fd_gpts_per_s", "value": v, "unit": "Gpts/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / max(1, len(res)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, None),
        "cpu_baseline": {"value": v, "unit": "Gpts/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, batch, shots_per_batch=None):
    surf = bool(getattr(args, "surf", False))
    return {"workload": "batched 2D shot RTM with illumination-normalised stacking" +
                        (", free surface and mirror receivers" if surf else ""),
            "surf_type": 1 if surf else 0, "rec_type": 1 if surf else 0,
            "grid": [NZ, NX], "spacing_m": D, "dt_s": DT, "ntaper": NTAPER, "snapi": SNAPI,
            "record_s": [3.0, 4.0], "aperture_m": [3000, 6000], "shot_spacing_m": SPACING,
            "survey_shots": NSHOT_SURVEY, "shots_per_step": batch,
            "shots_per_batch": shots_per_batch, "ricker_hz": F0,
            "l2": "inputs larger than L2 (snapshots of every shot in HBM)",
            "bytes_per_point": BYTES_PER_POINT}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shots-per-step", type=int, default=0,
                    help="shots per bench step (0: chosen by the autotuner)")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner: default launch shape, 16 shots per step unless "
                         "--shots-per-step says otherwise")
    ap.add_argument("--cpu-steps", type=int, default=0,
                    help="time samples of the CPU sample shot (0: its whole record)")
    ap.add_argument("--nt-cap", type=int, default=0, help="truncate records (debug)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precond-study", action="store_true",
                    help="run the learned-preconditioner FWI study instead of the RTM bench")
    ap.add_argument("--model3d", action="store_true",
                    help="time 3D modelling of one shot instead of the 2D RTM bench")
    ap.add_argument("--config5", type=int, default=0, metavar="NSHOT",
                    help="3D RTM of the first NSHOT shots of the 64-shot 400 x 400 x 200 survey "
                         "(12.5 m, dt 0.9 ms, 3 s) instead of the 2D bench")
    ap.add_argument("--surf", action="store_true",
                    help="the same RTM with a free surface (surf_type 1) and mirror receivers "
                         "(rec_type 1)")
    ap.add_argument("--revolve-study", action="store_true",
                    help="FWI gradient memory modes on the 1201 x 3401 grid: store-all against "
                         "binomial checkpointing with 32/64/128 state slots")
    ap.add_argument("--rho", action="store_true",
                    help="time 2D modelling with variable density (and without) on the "
                         "751 x 2301 grid instead of the RTM bench")
    ap.add_argument("--rho3d", action="store_true",
                    help="with --rho: 3D modelling on the 200 x 400 x 400 grid at 12.5 m "
                         "(the two-pass density operator on the point tiles)")
    ap.add_argument("--fwi-bench", action="store_true",
                    help="time one 80-shot FWI misfit and gradient evaluation on 601 x 1801")
    ap.add_argument("--cnn-bench", action="store_true",
                    help="time the preconditioner network's tensor-core kernels at 601 x 1801")
    ap.add_argument("--config4-study", action="store_true",
                    help="learned vs plain multiscale FWI on 601 x 1801 models (80 shots, "
                         "3/6/9 Hz) instead of the RTM bench")
    ap.add_argument("--c4-train", type=int, default=64, help="training models (301 x 901)")
    ap.add_argument("--c4-train-shots", type=int, default=20, help="shots per training model")
    ap.add_argument("--c4-evals", type=int, default=15, help="evaluations per stage (test)")
    ap.add_argument("--c4-train-evals", type=int, default=10,
                    help="evaluations per stage (training runs)")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch every time step directly (profiling runs: every launch timed)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.precond_study:
        return run_precond_study()
    if args.config4_study:
        return run_config4_study(args)
    if args.cnn_bench:
        return run_cnn_bench(args)
    if args.fwi_bench:
        return run_fwi_bench(args)
    if args.rho:
        return run_rho_bench(args)
    if args.model3d:
        return run_model3d(args)
    if args.revolve_study:
        return run_revolve_study(args)
    if args.config5:
        return run_config5(args)

    import torch

    import seismic_gb300 as sw
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    ctx = sw.Context(local)
    if args.no_graph:
        ctx.set_tuning(use_graph=0)
    g, vel, w, shots = make_workload(args.nt_cap or None)
    if args.surf:
        g.surf_type, g.rec_type = 1, 1
    # Shots of this rank: rank r takes every ws-th shot of the survey.
    from seismic_gb300 import dist as sdist
    mine = [shots[i] for i in sdist.shard(len(shots), rank, ws)]
    # Shots per step and launch shape: the autotuner (batch candidates
    # capped by what HBM admits at full record length, timed on truncated
    # records; then the launch shape at that batch), untimed.
    tune = None
    if not args.no_tune:
        from seismic_gb300 import autotune
        t0 = time.perf_counter()
        tune = autotune.tune_survey(ctx, g, vel, w, mine, steps=64)
        tune["tune_s"] = time.perf_counter() - t0
        if args.no_graph:
            ctx.set_tuning(use_graph=0)
        log(f"[rank {rank}] autotune: {tune}")
    B = args.shots_per_step or (tune["batch"] if tune else 16)
    nsteps = args.warmup + args.steps
    per_step = [mine[(k * B + q) % len(mine)] for k in range(nsteps) for q in range(B)]
    # Observed data: batched forward modelling on each shot's window (untimed).
    distinct = {}
    t0 = time.perf_counter()
    uniq = []
    for s in per_step:
        key = float(s["sou"][1])
        if key not in distinct:
            distinct[key] = None
            uniq.append(s)
    mj = sw.RTMJob(ctx, g, vel, w, [{"sou": s["sou"], "rec": s["rec"], "nt": s["nt"]} for s in uniq])
    mj.set_batch(B)
    for s, d in zip(uniq, mj.model()):
        distinct[float(s["sou"][1])] = d
    mj.close()
    log(f"[rank {rank}] modelled {len(uniq)} shots in {time.perf_counter() - t0:.1f}s")
    job_shots = [{"sou": s["sou"], "rec": s["rec"], "data": distinct[float(s["sou"][1])]}
                 for s in per_step]
    job = sw.RTMJob(ctx, g, vel, w, job_shots)
    job.set_batch(B)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # Warm-up steps.
    for k in range(args.warmup):
        job.run(k * B, B)
    barrier()
    # Timed region: inputs resident in HBM, no per-kernel events.
    ctx.reset_stats()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    t_start = time.perf_counter()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    torch.cuda.nvtx.range_push("timed")
    points = 0
    for k in range(args.warmup, nsteps):
        job.run(k * B, B)
        points += sum(shot_points(s) for s in per_step[k * B:(k + 1) * B])
    if ws > 1:
        # The exchange step: one sum of the stacked images over the ranks.
        sdist.allreduce_sum([job.result(normalised=False)[0]], device="cuda")
    ev1.record()
    torch.cuda.nvtx.range_pop()
    barrier()
    elapsed = time.perf_counter() - t_start
    ev_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    launches_timed_region = int(ctx.stats()["launches_total"])
    last_batch, _ = job.info()
    # Roofline pass: one more step with CUDA events bracketing the fused step
    # kernel (every 8th graph chunk), outside the timed region.
    ctx.reset_stats()
    ctx.set_profiling(True)
    job.run(args.warmup * B, B)
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    st = ctx.stats()
    secs = elapsed
    if ws > 1:
        secs = sdist.allreduce_max(secs, device="cuda")
        points_all = float(sdist.allreduce_sum([np.array([float(points)])], device="cuda")[0][0])
    else:
        points_all = float(points)
    value = points_all / secs / 1e9
    # Roofline of the fused step kernel from the roofline pass's events.
    peak, peak_kind = measured_peak()
    kern_s = st["step_kernel_ms"] / 1e3
    nl = max(1, st["step_kernel_timed"])
    achieved = (st["step_bytes"] / nl) / (kern_s / nl) / 1e9 if kern_s > 0 else None
    # DRAM traffic per launch: the ratio of ncu-measured DRAM bytes to
    # algorithmic bytes over every fused-kernel launch of a smaller RTM batch
    # (profiles/step_kernel_traffic.json) times this run's algorithmic bytes.
    algo_per_launch = st["step_bytes"] / nl
    traffic = None
    prof_json = os.path.join(ROOT, "profiles", "step_kernel_traffic.json")
    if os.path.exists(prof_json):
        try:
            traffic = float(json.load(open(prof_json))["dram_per_algorithmic"]) * algo_per_launch
        except Exception:
            traffic = None
    # End to end through the public API with host buffers: the timed steps'
    # shots again, through a new job (model, wavelet and traces copied from
    # pinned host memory, the images read back).
    e2e_line = None
    if rank == 0:
        sel = job_shots[args.warmup * B:nsteps * B]
        pin = lambda a: _pinned(torch, a)
        hshots = [{"sou": s["sou"], "rec": s["rec"], "data": pin(s["data"])} for s in sel]
        hvel = pin(vel)
        hw = pin(w)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        j2 = sw.RTMJob(ctx, g, hvel, hw, hshots)
        j2.set_batch(B)
        j2.run()
        im, il, nm = j2.result(normalised=True)
        j2.close()
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        pts_e2e = sum(shot_points(s) for s in per_step[args.warmup * B:nsteps * B])
        h2d = hvel.nbytes + hw.nbytes + sum(s["data"].nbytes + s["rec"].nbytes for s in hshots)
        d2h = im.nbytes + il.nbytes + nm.nbytes
        e2e_line = {"value": pts_e2e / e2e_s / 1e9, "unit": "Gpts/s",
                    "h2d_bytes_per_step": int(h2d) // args.steps,
                    "d2h_bytes_per_step": int(d2h) // args.steps}
    # CPU baseline (rank 0, N=1 only): the oracle's RTM of the first two
    # shots of the first timed batch with the same data, which also checks
    # the GPU's image of those shots.
    cpu, parity = None, None
    if rank == 0 and ws == 1 and not args.no_cpu:
        k0 = args.warmup * B
        psh = job_shots[k0:k0 + min(2, B)]
        r, parity = cpu_parity_sample(ctx, g, vel, w, psh)
        cpu = {"value": r["points"] / r["seconds"] / 1e9, "unit": "Gpts/s", "cores": cpu_threads(),
               "kind": "port",
               "sample": f"oracle stacked RTM (forward + backward, whole records) of {len(psh)} "
                         f"shots of the first timed batch with the GPU's data "
                         f"({r['seconds']:.1f} s)"}
    if rank == 0:
        line = {
            "metric": "fd_gpts_per_s", "value": value, "unit": "Gpts/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded faulted layered model, data modelled by the engine)",
            "config": workload_config(args, B, last_batch),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "peak_kind": peak_kind, "kernel": "k_bstep2d_t (fused stencil + time update, pipelined 2D tiles)",
                         "avg_launch_ms": (st["step_kernel_ms"] / nl),
                         "algorithmic_bytes_per_launch": algo_per_launch,
                         "launches_timed": st["step_kernel_timed"]},
            "cpu_baseline": cpu, "parity": parity, "e2e": e2e_line, "clocks": clk,
            "gpu_launches": launches_timed_region,
            "timed_event_ms": ev_ms,
            "autotune": tune,
        }
        print(json.dumps(line), flush=True)
    job.close()
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_model3d(args) -> int:
    """3D modelling of one shot (sw_modeling; the TMA-pipelined 3D step
    kernel): a 200 x 400 x 400 model at 12.5 m, 2500 receivers, nt steps.
    Prints its own JSON line; the headline bench stays the 2D RTM."""
    import torch

    import seismic_gb300 as sw
    from seismic_gb300 import synth
    torch.cuda.set_device(0)
    ctx = sw.Context(0)
    nz, nx, ny, d, dt = 200, 400, 400, 12.5, 9e-4
    nt = args.nt_cap or 400
    g = sw.make_genpar(nz, nx, ny, dz=d, dx=d, dy=d, dt=dt, nt=nt, ntaper=20, lsinc=7,
                       snapi=4, twoD=False, fmax=20.0)
    z = np.arange(nz)[None, None, :] * d
    vel = np.ascontiguousarray(np.broadcast_to(1500.0 + 1.0 * z, (ny, nx, nz)), np.float32)
    sou = np.array([25.0, nx * d / 2, ny * d / 2], np.float32)
    rx, ry = np.meshgrid(np.arange(10, nx - 10, 8) * d, np.arange(10, ny - 10, 8) * d,
                         indexing="ij")
    rec = np.zeros((rx.size, 3), np.float32)
    rec[:, 0], rec[:, 1], rec[:, 2] = 12.5, rx.ravel(), ry.ravel()
    w = synth.ricker(10.0, dt, nt)
    for _ in range(max(1, args.warmup)):
        ctx.modeling(g, vel, sou, w, rec)
    ctx.reset_stats()
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("timed")
    for _ in range(args.steps):
        ctx.modeling(g, vel, sou, w, rec)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    clk = clocks.stop()
    st = ctx.stats()
    points = float(st["points_updated"])
    ctx.reset_stats()
    ctx.set_profiling(True)
    ctx.modeling(g, vel, sou, w, rec)
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    sp = ctx.stats()
    peak, peak_kind = measured_peak()
    nl = max(1, sp["step_kernel_timed"])
    kern_s = sp["step_kernel_ms"] / 1e3
    achieved = (sp["step_bytes"] / nl) / (kern_s / nl) / 1e9 if kern_s > 0 else None
    line = {
        "metric": "fd_gpts_per_s_3d_modeling", "value": points / secs / 1e9, "unit": "Gpts/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (linear velocity gradient)",
        "config": {"workload": "3D modelling of one shot through sw_modeling (host buffers)",
                   "grid": [nz, nx, ny], "spacing_m": d, "dt_s": dt, "nt": nt,
                   "ntaper": 20, "receivers": int(rec.shape[0])},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "peak_kind": peak_kind,
                     "kernel": "k_bstep3d_t (fused stencil + time update, TMA plane pipeline)",
                     "avg_launch_ms": sp["step_kernel_ms"] / nl,
                     "algorithmic_bytes_per_launch": sp["step_bytes"] / nl},
        "clocks": clk, "gpu_launches": int(st["launches_total"]),
    }
    print(json.dumps(line))
    return 0


def run_rho_bench(args) -> int:
    """Variable density: 2D modelling of one shot on the full 751 x 2301
    model at 4 m (the RTM bench's grid and dt, 2000 steps, 2301 receivers)
    through sw_propagate with a density model (withRho: the one-pass
    staggered operator, k_brho2d) and, for scale, the same run without it.
    With --rho3d: 3D modelling on the 200 x 400 x 400 grid at 12.5 m (400
    steps, 2304 receivers), where the density operator is the gradient
    pass plus the point-tile step.  One JSON line with the density step
    kernel's roofline."""
    import torch

    import seismic_gb300 as sw
    from seismic_gb300 import synth
    torch.cuda.set_device(0)
    ctx = sw.Context(0)
    rng = np.random.default_rng(3)
    if args.rho3d:
        nz, nx, ny, d, dt = 200, 400, 400, 12.5, 9e-4
        nt = args.nt_cap or 400
        g = sw.make_genpar(nz, nx, ny, dz=d, dx=d, dy=d, dt=dt, nt=nt, ntaper=20, lsinc=7,
                           snapi=4, twoD=False, fmax=20.0)
        z = np.arange(nz)[None, None, :] * d
        vel = np.ascontiguousarray(np.broadcast_to(1500.0 + 1.0 * z, (ny, nx, nz)), np.float32)
        rho = np.ascontiguousarray(1.8 + 0.0004 * z + 0.1 * rng.random(vel.shape), np.float32)
        sou = np.array([25.0, nx * d / 2, ny * d / 2], np.float32)
        rx, ry = np.meshgrid(np.arange(10, nx - 10, 8) * d, np.arange(10, ny - 10, 8) * d,
                             indexing="ij")
        rec = np.zeros((rx.size, 3), np.float32)
        rec[:, 0], rec[:, 1], rec[:, 2] = 12.5, rx.ravel(), ry.ravel()
        w = sw.rho_wavelet(synth.ricker(10.0, dt, nt), 7)
        workload = ("3D modelling of one shot with variable density through sw_propagate "
                    "(host buffers)")
        grid, kernel = [nz, nx, ny], ("k_bstep<false> after k_brho_grad (two-pass density "
                                      "operator on the point tiles, 40 B per point)")
    else:
        c = synth.CONFIG2
        nt = args.nt_cap or 2000
        nz, nx, d, dt = c["nz"], c["nx"], c["d"], c["dt"]
        g = sw.make_genpar(nz, nx, 1, dz=d, dx=d, dt=dt, nt=nt, ntaper=c["ntaper"], lsinc=7,
                           snapi=4)
        vel = synth.layered_faulted(nz, nx, d, seed=3)
        rho = np.ascontiguousarray(1.8 + 0.0004 * np.arange(nz)[None, :] * d +
                                   0.1 * rng.random(vel.shape), np.float32)
        sou = np.array([2 * d, nx * d / 2, 0.0], np.float32)
        rec = np.zeros((nx, 3), np.float32)
        rec[:, 0], rec[:, 1] = 2 * d, np.arange(nx) * d
        w = sw.rho_wavelet(synth.ricker(20.0, dt, nt), 7)
        workload = ("2D modelling of one shot with variable density through sw_propagate "
                    "(host buffers)")
        grid, kernel = [nz, nx], ("k_brho2d (one-pass staggered gradient, divergence and time "
                                  "update, 32 B per point)")
    desc = sw.SwPropDesc()
    desc.g = g
    desc.tmin, desc.tmax, desc.tstep = 1, nt, 1
    desc.fd_scheme = sw.FD_FORWARD
    desc.injection, desc.extraction = sw.INJ_SINC, sw.EXT_SINC
    data = np.zeros((rec.shape[0], nt), np.float32)

    def run(with_rho):
        ctx.propagate(desc, vel, sou[None], w[None], rec, data,
                      rho=rho if with_rho else None)

    out = {}
    clk = None
    for with_rho in (True, False):
        for _ in range(max(1, args.warmup)):
            run(with_rho)
        ctx.reset_stats()
        if with_rho:
            clocks = ClockSampler(0)
            clocks.start()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run(with_rho)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        if with_rho:
            clk = clocks.stop()
        st = ctx.stats()
        out[with_rho] = (float(st["points_updated"]) / secs / 1e9, secs / args.steps,
                         int(st["launches_total"]))
    # The density step kernel's duration from CUDA events around it in one
    # more (untimed) run.
    ctx.reset_stats()
    ctx.set_profiling(True)
    run(True)
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    sp = ctx.stats()
    peak, peak_kind = measured_peak()
    nl = max(1, sp["step_kernel_timed"])
    kern_s = sp["step_kernel_ms"] / 1e3
    achieved = (sp["step_bytes"] / nl) / (kern_s / nl) / 1e9 if kern_s > 0 else None
    line = {
        "metric": "fd_gpts_per_s_%s_rho_modeling" % ("3d" if args.rho3d else "2d"),
        "value": out[True][0], "unit": "Gpts/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": out[True][1] * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": ("synthetic (linear velocity gradient; density 1.8-2.9 g/cc)" if args.rho3d
                 else "synthetic (seeded layered, faulted model; density 1.8-2.2 g/cc)"),
        "config": {"workload": workload, "grid": grid, "spacing_m": d, "dt_s": dt, "nt": nt,
                   "receivers": int(rec.shape[0])},
        "constant_density_gpts_per_s": out[False][0],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "peak_kind": peak_kind,
                     "kernel": kernel,
                     "avg_launch_ms": sp["step_kernel_ms"] / nl,
                     "algorithmic_bytes_per_launch": sp["step_bytes"] / nl},
        "clocks": clk, "gpu_launches": out[True][2],
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def run_config5(args) -> int:
    """3D RTM through the multi-shot job: the 400 (x) x 400 (y) x 200 (z)
    model at 12.5 m (25 dipping layers, 4 faults, salt at 4500 m/s), dt
    0.9 ms, 3333 steps, 15 Hz, 2500 receivers over the model, snapshots every
    4 steps in HBM; the first NSHOT of the 64 shots, admitted into batches
    by their HBM footprint (about 107 GB of snapshots per shot).  Reports
    Gpts/s, the shots per batch, the 3D step kernel's roofline from a
    profiled batch, and a CPU sample (the oracle's RTM of one shot window
    over a bounded number of steps)."""
    import torch

    import seismic_gb300 as sw
    from oracle import bind as oracle
    from seismic_gb300 import synth
    torch.cuda.set_device(0)
    ctx = sw.Context(0)
    t0 = time.perf_counter()
    c5 = synth.config5(args.nt_cap or None)
    g, vel, w = c5["g"], c5["vel"], c5["wavelet"]
    shots = c5["shots"][:args.config5]
    log(f"config-5 model built in {time.perf_counter() - t0:.1f}s")
    ap = 6000.0
    mj = sw.RTMJob(ctx, g, vel, w, shots, aperture_x=ap, aperture_y=ap)
    t0 = time.perf_counter()
    data = mj.model()
    mj.close()
    log(f"modelled {len(shots)} shots in {time.perf_counter() - t0:.1f}s")
    job_shots = [{"sou": s["sou"], "rec": s["rec"], "data": d} for s, d in zip(shots, data)]
    job = sw.RTMJob(ctx, g, vel, w, job_shots, aperture_x=ap, aperture_y=ap)
    job.set_batch(64, 0.85)
    job.run(0, min(2, len(shots)))                  # warm-up (arena, graphs)
    job.reset()
    ctx.reset_stats()
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    job.run()
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    clk = clocks.stop()
    st = ctx.stats()
    batch, _ = job.info()
    # Roofline pass: one batch again with CUDA events around the step kernel.
    ctx.reset_stats()
    ctx.set_profiling(True)
    job.run(0, batch)
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    sp = ctx.stats()
    job.close()
    peak, peak_kind = measured_peak()
    nl = max(1, sp["step_kernel_timed"])
    kern_s = sp["step_kernel_ms"] / 1e3
    achieved = (sp["step_bytes"] / nl) / (kern_s / nl) / 1e9 if kern_s > 0 else None
    # CPU sample: the oracle's 3D RTM of the first shot's window over 60 steps.
    cpu = None
    if not args.no_cpu:
        win, gw = sw.shot_window(g, ap, ap, shots[0]["sou"], shots[0]["rec"])
        gw.nt = 60
        vwin = sw.window_extract(g, win, vel)
        dcut = np.ascontiguousarray(data[0][:, :60])
        t0 = time.perf_counter()
        oracle.rtm(gw, vwin, shots[0]["sou"], w[:60], shots[0]["rec"], dcut)
        cs = time.perf_counter() - t0
        pts = ((gw.nz + 2 * gw.ntaper) * (gw.nx + 2 * gw.ntaper) * (gw.ny + 2 * gw.ntaper) *
               60 * 2)
        cpu = {"value": pts / cs / 1e9, "unit": "Gpts/s", "cores": cpu_threads(), "kind": "port",
               "sample": f"oracle 3D RTM of one shot window, 60 of {g.nt} steps ({cs:.1f} s)"}
    line = {
        "metric": "fd_gpts_per_s_3d_rtm", "value": st["points_updated"] / secs / 1e9,
        "unit": "Gpts/s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak", "dtype": "f32",
        "vs_baseline": None,
        "data": "synthetic (seeded 3D layered, faulted model with salt; data modelled by the "
                "engine)",
        "config": {"workload": "3D shot RTM with illumination-normalised stacking",
                   "grid": [g.nz, g.nx, g.ny], "spacing_m": g.dx, "dt_s": g.dt, "nt": g.nt,
                   "snapi": g.snapi, "ntaper": g.ntaper, "shots": len(shots),
                   "survey_shots": 64, "receivers": int(shots[0]["rec"].shape[0]),
                   "aperture_m": ap, "shots_per_batch": batch,
                   "l2": "inputs larger than L2 (snapshots of every shot in HBM)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "peak_kind": peak_kind,
                     "kernel": "k_bstep3d_t (fused stencil + time update + imaging condition, "
                               "TMA plane pipeline; Higdon lines in the edge kernels)",
                     "avg_launch_ms": sp["step_kernel_ms"] / nl,
                     "algorithmic_bytes_per_launch": sp["step_bytes"] / nl,
                     "launches_timed": sp["step_kernel_timed"]},
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(st["launches_total"]),
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def run_revolve_study(args) -> int:
    """FWI gradient of one shot on the 1201 x 3401 grid at 6.25 m (dt 0.5 ms,
    10000 steps unless --nt-cap): store-all snapshots in HBM against the
    binomial checkpoint schedule with 32, 64 and 128 state slots (segments
    of 10 snapshots).  Per mode: device memory of the snapshot store, forward
    and backward time steps (recompute factor = forward steps / nt), wall
    time per gradient, and whether misfit and gradient equal store-all's bit
    for bit.  One JSON line."""
    import torch

    import seismic_gb300 as sw
    from seismic_gb300 import synth
    torch.cuda.set_device(0)
    ctx = sw.Context(0)
    c3 = synth.config3(nt=args.nt_cap or None)
    g, vb, ref, rec = c3["g"], c3["vel"], c3["ref"], c3["rec"]
    w = c3["wavelet"]
    nt = g.nt
    vtrue = (vb * (1.0 + ref)).astype(np.float32)
    sou = c3["shots"][len(c3["shots"]) // 2]
    desc = sw.SwFwiDesc()
    desc.g = g
    desc.aperture_x, desc.aperture_y, desc.illu_pow = 1e5, 0.0, 1.0
    desc.smooth_rect1 = desc.smooth_rect2 = desc.smooth_rect3 = 1
    shot = {"sou": sou, "rec": rec, "dobs": np.zeros((rec.shape[0], nt), np.float32)}
    _, _, _, res = ctx.fwi_fct_gdt(desc, vtrue, w, [shot], want_resid=True)
    shot["dobs"] = -res[0]                       # data of the true model
    nw = g.nz * g.nx
    pad = (g.nz + 2 * g.ntaper + 8) * (g.nx + 2 * g.ntaper + 8)
    ntsnap = nt // g.snapi
    K = 10
    rows, base = [], None
    for slots in (None, 32, 64, 128):
        desc.checkpoint_snaps = 0 if slots is None else K
        desc.revolve_slots = 0 if slots is None else slots
        ctx.fwi_fct_gdt(desc, vb, w, [shot])     # warm-up (arena, graphs)
        ctx.reset_stats()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f, grad, _ = ctx.fwi_fct_gdt(desc, vb, w, [shot])
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        st = ctx.stats()
        if slots is None:
            mem = ntsnap * nw * 4
            base = (f, grad)
        else:
            mem = (slots + 1) * 4 * pad * 4 + (K + 2) * nw * 4
        rows.append({"mode": "store-all" if slots is None else f"revolve-{slots}",
                     "snapshot_store_gb": mem / 1e9,
                     "steps_forward": int(st["steps_forward"]),
                     "steps_backward": int(st["steps_backward"]),
                     "recompute_factor": st["steps_forward"] / nt,
                     "segment_advances": int(st["ckpt_advances"]),
                     "seconds_per_gradient": secs,
                     "gpts_per_s": st["points_updated"] / secs / 1e9,
                     "bitexact_vs_store_all": bool(f == base[0] and np.array_equal(grad, base[1]))})
        log(json.dumps(rows[-1]))
    print(json.dumps({"study": "FWI gradient memory modes", "grid": [g.nz, g.nx],
                      "spacing_m": g.dx, "dt_s": g.dt, "nt": nt, "snapi": g.snapi,
                      "segment_snapshots": K, "receivers": int(rec.shape[0]), "rows": rows}),
          flush=True)
    ctx.close()
    return 0


def run_precond_study() -> int:
    """Learned-preconditioned vs plain L-BFGS FWI on seeded 60 x 180 models
    (network trained on plain runs over 12 other seeds); one JSON line."""
    import seismic_gb300 as sw
    from seismic_gb300 import precond
    ctx = sw.Context(0)
    r = precond.run_study(ctx, train_seeds=tuple(range(1000, 1012)), test_seeds=(4, 5, 6),
                          epochs=400, f0=5.0, smooth_m=120.0,
                          learned_kw={"max_learned": 3, "c1": 0.1})
    for row in r["tests"]:
        row.pop("plain_curve")
        row.pop("learned_curve")
    print(json.dumps({"study": "learned vs plain L-BFGS FWI", **r}), flush=True)
    ctx.close()
    return 0


def run_config4_study(args) -> int:
    """Learned-preconditioned vs plain L-BFGS multiscale FWI at the 601 x 1801
    benchmark size (80 shots, 3/6/9 Hz stages), the network trained on plain
    runs over --c4-train seeded 301 x 901 models; one JSON line."""
    import seismic_gb300 as sw
    from seismic_gb300 import precond
    ctx = sw.Context(0)
    r = precond.run_config4_study(ctx, n_train=args.c4_train, train_nshot=args.c4_train_shots,
                                  evals_per_stage=args.c4_evals,
                                  train_evals_per_stage=args.c4_train_evals,
                                  learned_kw={"max_learned": 3, "c1": 0.1}, log=log)
    print(json.dumps({"study": "learned vs plain L-BFGS multiscale FWI", **r}), flush=True)
    ctx.close()
    return 0


def run_fwi_bench(args) -> int:
    """One FWI misfit and gradient evaluation (compute_fct_gdt: forward
    modelling, residual, adjoint propagation with the AFWI imaging
    condition, every snapshot in HBM) of the learned-preconditioner study's
    test survey: 601 x 1801 model at 10 m, 80 shots, 4 s at dt 0.9 ms,
    6 Hz Ricker, start model smoothed by 250 m; observed data modelled on
    the true model.  Shots run in HBM-admitted batches.  One JSON line."""
    import torch

    import seismic_gb300 as sw
    from seismic_gb300 import precond
    torch.cuda.set_device(0)
    ctx = sw.Context(0)
    cfg = precond.CONFIG4
    sv = precond._stage_survey(ctx, 7, cfg["test"], 6.0, cfg["nshot"], cfg)
    x = sv.v0.astype(np.float32)
    for _ in range(max(1, args.warmup)):
        ctx.fwi_fct_gdt(sv.desc, x, sv.wavelet, sv.shots)
    ctx.reset_stats()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.fwi_fct_gdt(sv.desc, x, sv.wavelet, sv.shots)
    secs = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    st = ctx.stats()
    line = {
        "metric": "fwi_gradient_gpts_per_s", "value": st["points_updated"] / args.steps / secs / 1e9,
        "unit": "Gpts/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak", "dtype": "f32",
        "vs_baseline": None, "data": "synthetic (seeded layered, faulted model; data modelled "
                                     "by the engine)",
        "config": {"workload": "FWI misfit and gradient of 80 shots (store-all snapshots)",
                   "grid": list(cfg["test"]), "spacing_m": cfg["d"], "dt_s": cfg["dt"],
                   "record_s": cfg["t"], "shots": cfg["nshot"], "ricker_hz": 6.0},
        "seconds_per_evaluation": secs,
        "solves_per_second": 2 * cfg["nshot"] / secs,
        "clocks": clk, "gpu_launches": int(st["launches_total"]) // args.steps,
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def run_cnn_bench(args) -> int:
    """The preconditioner network at the FWI benchmark's test size (601 x 1801
    image, 2 -> 32 -> 32 -> 32 -> 1 channels): inference and gradient passes
    per second through the public API, and the event-timed roofline of the
    tensor-core convolution and weight-gradient kernels (algorithmic bytes:
    BF16 activations read once, outputs written once; FLOPs of the real
    channels).  One JSON line."""
    import torch

    import seismic_gb300 as sw
    torch.cuda.set_device(0)
    ctx = sw.Context(0)
    nz, nx, ch = 601, 1801, (2, 32, 32, 32, 1)
    rng = np.random.default_rng(8)
    x = rng.standard_normal((1, 2, nx, nz)).astype(np.float32)
    t = rng.standard_normal((1, nx, nz)).astype(np.float32)
    net = sw.CNN(ctx, ch, seed=0)
    for _ in range(max(args.warmup, 1)):
        net.forward(x[0])
        net.gradient(x, t)
    reps = max(args.steps, 1)
    ctx.reset_stats()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(reps):
        net.forward(x[0])
    t_fwd = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        net.gradient(x, t)
    t_grad = (time.perf_counter() - t0) / reps
    clk = clocks.stop()
    launches = int(ctx.stats()["launches_total"])
    # Roofline pass: one gradient call with every tensor-core launch timed.
    ctx.reset_stats()
    ctx.set_profiling(True)
    net.gradient(x, t)
    ctx.set_profiling(False)
    st = ctx.stats()
    net.close()
    ctx.close()
    peak, peak_kind = measured_peak()
    tf_peak = None
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        tf_peak = mp.get("bf16_tflops")
    except Exception:
        pass
    secs = st["cnn_conv_ms"] / 1e3
    gbs = st["cnn_conv_bytes"] / secs / 1e9 if secs > 0 else None
    tfs = st["cnn_conv_flops"] / secs / 1e12 if secs > 0 else None
    line = {
        "metric": "cnn_gradient_passes_per_s", "value": 1.0 / t_grad, "unit": "passes/s",
        "n_gpus": 1, "steps": reps, "warmup": args.warmup, "ms_per_step": t_grad * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded normal inputs and targets)",
        "config": {"workload": "preconditioner network forward + backward on one image",
                   "image": [nz, nx], "channels": list(ch),
                   "l2": "activations (69 MB per 32-channel tensor) mostly L2-resident"},
        "forward_ms": t_fwd * 1e3,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                     "frac": gbs / peak if gbs else None, "peak_kind": peak_kind,
                     "tensor_tflops": tfs, "tensor_peak_tflops": tf_peak,
                     "tensor_frac": (tfs / tf_peak) if (tfs and tf_peak) else None,
                     "kernel": "k_conv_tma + k_wgrad_umma (tcgen05, TMA-fed)",
                     "launches_timed": st["cnn_conv_timed"],
                     "avg_launch_ms": st["cnn_conv_ms"] / max(1, st["cnn_conv_timed"]),
                     "algorithmic_bytes": st["cnn_conv_bytes"],
                     "flops": st["cnn_conv_flops"]},
        "clocks": clk, "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)
    return 0


def _pinned(torch, a: np.ndarray) -> np.ndarray:
    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
    t.numpy()[...] = a
    return t.numpy()


if __name__ == "__main__":
    sys.exit(main())

"""Autotuner for the fused step kernel's launch shape, the graph chunk and
the number of shots per launch.

Candidates are timed on a truncated copy of the real batch (same windows,
same number of shots in flight, a few dozen time steps of both the forward
and the backward phase); the fastest is cached per (device, padded-grid
bucket, shots per batch) in a JSON file under the user's cache directory.
With `batch="auto"` the shots per launch are chosen first (each candidate
batch size runs the same sample of shots, in as many launches as it needs,
with the current launch shape), then the launch shape at that batch size.
Timing is injected so that the selection logic can be exercised without a
GPU.
"""
from __future__ import annotations

import json
import os
import time
from typing import Callable, Iterable

DEFAULT_CACHE = os.path.join(os.environ.get("XDG_CACHE_HOME", os.path.expanduser("~/.cache")),
                             "seismic_gb300", "tuning.json")


def candidates(two_d: bool = True) -> list[dict]:
    out = []
    for chunk in (16, 32):
        out.append({"step_kernel": 0, "tile_z": 64, "tile_x": 64, "tile_y": 32,
                    "graph_chunk": chunk, "use_graph": 1})
        if two_d:
            # TMA-staged tiles: 2 CTAs per SM (2), warp-specialised (3) and
            # two steps per launch (4).
            for k in (2, 3, 4):
                out.append({"step_kernel": k, "tile_z": 64, "tile_x": 64, "tile_y": 32,
                            "graph_chunk": chunk, "use_graph": 1})
            for tz in (32, 64, 128):
                for tx in (32, 64, 128, 256):
                    out.append({"step_kernel": 1, "tile_z": tz, "tile_x": tx, "tile_y": 32,
                                "graph_chunk": chunk, "use_graph": 1})
        else:
            for ty in (8, 16, 32, 64):
                out.append({"step_kernel": 1, "tile_z": 64, "tile_x": 64, "tile_y": ty,
                            "graph_chunk": chunk, "use_graph": 1})
    return out


def bucket(n: int, step: int = 64) -> int:
    return (n + step - 1) // step * step


def cache_key(device: str, n1p: int, n2p: int, n3p: int, batch: int) -> str:
    return f"{device}|{bucket(n1p)}x{bucket(n2p)}x{bucket(n3p, 8)}|b{batch}"


def load_cache(path: str = DEFAULT_CACHE) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path: str = DEFAULT_CACHE) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def select(cands: Iterable[dict], time_fn: Callable[[dict], float], repeats: int = 2) -> tuple[dict, list]:
    """Returns the candidate with the smallest best-of-`repeats` time."""
    results = []
    for c in cands:
        try:
            t = min(time_fn(c) for _ in range(repeats))
        except Exception as e:  # a candidate the device rejects is skipped
            results.append((c, float("inf"), repr(e)))
            continue
        results.append((c, t, None))
    ok = [r for r in results if r[1] != float("inf")]
    if not ok:
        raise RuntimeError("no tuning candidate ran: " + "; ".join(str(r[2]) for r in results))
    best = min(ok, key=lambda r: r[1])
    return best[0], results


BATCH_CANDIDATES = (1, 2, 4, 8, 16, 32, 64)


def batch_candidates(nshots: int, cands: Iterable[int] = BATCH_CANDIDATES) -> list[int]:
    """Batch sizes worth timing for a survey of `nshots` shots: those below
    the shot count, plus the shot count itself when it is below the largest
    candidate (a batch larger than the survey runs the same launch)."""
    out = sorted({b for b in cands if b < nshots} | ({nshots} if nshots <= max(cands) else set()))
    return out or [1]


def select_batch(batches: Iterable[int], time_fn: Callable[[int], float],
                 repeats: int = 2) -> tuple[int, list]:
    """The batch size whose run of the same shot sample is fastest (ties go
    to the smaller batch, which holds less memory)."""
    best, res = select([{"batch": b} for b in sorted(batches)], lambda c: time_fn(c["batch"]),
                       repeats)
    return best["batch"], res


def _sample(shots, count, steps):
    import numpy as np
    return [{"sou": shots[i % len(shots)]["sou"], "rec": shots[i % len(shots)]["rec"],
             "data": np.ascontiguousarray(np.asarray(shots[i % len(shots)]["data"])[:, :steps])}
            for i in range(count)]


def _device_name(ctx, device_name):
    if device_name is not None:
        return device_name
    try:
        import torch
        return torch.cuda.get_device_name(ctx_device(ctx))
    except Exception:
        return "cuda"


def tune_batch(ctx, model, vel, wavelet, shots, steps: int = 48,
               cands: Iterable[int] = BATCH_CANDIDATES, cache_path: str | None = DEFAULT_CACHE,
               device_name: str | None = None, force: bool = False) -> dict:
    """Chooses the shots per launch for the RTM job of `shots` with ctx's
    current launch shape.  Every candidate runs the same sample (the largest
    candidate's worth of shots, cycling through `shots`), so the times
    compare whole-sample throughput."""
    import numpy as np

    import seismic_gb300 as sw
    batches = batch_candidates(len(shots), cands)
    sample = _sample(shots, max(batches), steps)
    g = sw.SwGenpar.from_buffer_copy(model)
    g.nt = steps
    n1p = g.nz + 2 * g.ntaper + 8
    widths = [int(np.ptp(np.asarray(s["rec"])[:, 1]) / g.dx) + 1 for s in sample]
    n2p = max(widths) + 2 * g.ntaper + 8
    n3p = 1 if g.twoD else g.ny + 2 * g.ntaper + 8
    key = cache_key(_device_name(ctx, device_name), n1p, n2p, n3p, len(shots)) + "|batch"
    cache = load_cache(cache_path) if cache_path else {}
    if key in cache and not force:
        return cache[key]
    job = sw.RTMJob(ctx, g, vel, wavelet[:steps], sample)

    def time_fn(b):
        job.set_batch(b)
        job.run(0, len(sample))          # warm (graph capture, arena)
        t0 = time.perf_counter()
        job.run(0, len(sample))
        return time.perf_counter() - t0

    try:
        best, results = select_batch(batches, time_fn)
    finally:
        job.close()
    entry = {"batch": best, "seconds": {str(r[0]["batch"]): r[1] for r in results},
             "shots_timed": len(sample), "steps": steps}
    if cache_path:
        cache[key] = entry
        save_cache(cache, cache_path)
    return entry


def tune_rtm(ctx, model, vel, wavelet, shots, steps: int = 48, batch: int | str | None = None,
             cache_path: str | None = DEFAULT_CACHE, device_name: str | None = None,
             force: bool = False) -> dict:
    """Tunes ctx for the RTM job of `shots` and applies the winner.  `batch`
    is the shots per launch (default: all of `shots`); "auto" chooses it
    first (tune_batch) and returns it in the entry's "batch"."""
    import numpy as np

    import seismic_gb300 as sw
    chosen = None
    if batch == "auto":
        chosen = tune_batch(ctx, model, vel, wavelet, shots, steps=steps, cache_path=cache_path,
                            device_name=device_name, force=force)
        batch = chosen["batch"]
    batch = min(batch or len(shots), len(shots))
    sample = [{"sou": s["sou"], "rec": s["rec"],
               "data": np.ascontiguousarray(np.asarray(s["data"])[:, :steps])} for s in shots[:batch]]
    g = sw.SwGenpar.from_buffer_copy(model)
    g.nt = steps
    n1p = g.nz + 2 * g.ntaper + 8
    widths = [int(np.ptp(np.asarray(s["rec"])[:, 1]) / g.dx) + 1 for s in sample]
    n2p = max(widths) + 2 * g.ntaper + 8
    n3p = 1 if g.twoD else g.ny + 2 * g.ntaper + 8
    key = cache_key(_device_name(ctx, device_name), n1p, n2p, n3p, batch)
    cache = load_cache(cache_path) if cache_path else {}
    if key in cache and not force:
        ctx.set_tuning(**cache[key]["tuning"])
        return dict(cache[key], batch=batch) if chosen else cache[key]
    job = sw.RTMJob(ctx, g, vel, wavelet[:steps], sample)
    job.set_batch(batch)

    def time_fn(c):
        ctx.set_tuning(**c)
        job.run(0, len(sample))          # warm (graph capture, arena)
        t0 = time.perf_counter()
        job.run(0, len(sample))
        return time.perf_counter() - t0

    try:
        best, results = select(candidates(bool(g.twoD)), time_fn)
    finally:
        job.close()
    ctx.set_tuning(**best)
    entry = {"tuning": best, "seconds": min(r[1] for r in results),
             "tried": len(results), "steps": steps}
    if cache_path:
        cache[key] = entry
        save_cache(cache, cache_path)
    return dict(entry, batch=batch) if chosen else entry


def tune_survey(ctx, model, vel, wavelet, shots, steps: int = 64, mem_fraction: float = 0.85,
                cache_path: str | None = DEFAULT_CACHE, device_name: str | None = None,
                force: bool = False) -> dict:
    """Shots per launch and launch shape for the RTM of a whole survey.

    `shots` carry "sou", "rec" and "nt" (full record length); "data" is not
    needed.  The batch candidates are capped by what one batch of the
    survey's full-length records admits in device memory now
    (sw_rtm_job_admit with max_shots 64), and that cap is a candidate
    itself; each candidate is timed on the first shots' truncated records
    modelled by the engine (`steps` samples), then the launch shape is tuned
    at the chosen batch (tune_rtm).  Applies the winning launch shape to
    ctx and returns {"batch", "admit_cap", "tuning", "batch_seconds",
    "seconds", "tried", "steps"}."""
    import numpy as np

    import seismic_gb300 as sw
    g = sw.SwGenpar.from_buffer_copy(model)
    full = sw.RTMJob(ctx, g, vel, wavelet, [{"sou": s["sou"], "rec": s["rec"], "nt": s["nt"]}
                                            for s in shots])
    try:
        full.set_batch(max(BATCH_CANDIDATES), mem_fraction)
        cap = full.admit(0)
    finally:
        full.close()
    cands = sorted({b for b in BATCH_CANDIDATES if b <= cap} | {min(cap, len(shots))})
    nsample = max(cands)
    gs = sw.SwGenpar.from_buffer_copy(model)
    gs.nt = steps
    first = [shots[i % len(shots)] for i in range(nsample)]
    mj = sw.RTMJob(ctx, gs, vel, np.ascontiguousarray(wavelet[:steps]),
                   [{"sou": s["sou"], "rec": s["rec"], "nt": steps} for s in first])
    try:
        mj.set_batch(nsample)
        data = mj.model()
    finally:
        mj.close()
    sample = [{"sou": s["sou"], "rec": s["rec"], "data": d} for s, d in zip(first, data)]
    b = tune_batch(ctx, gs, vel, wavelet, sample, steps=steps, cands=cands,
                   cache_path=cache_path, device_name=device_name, force=force)
    t = tune_rtm(ctx, gs, vel, wavelet, sample, steps=steps, batch=b["batch"],
                 cache_path=cache_path, device_name=device_name, force=force)
    return {"batch": b["batch"], "admit_cap": cap, "tuning": t["tuning"],
            "batch_seconds": b["seconds"], "seconds": t["seconds"], "tried": t["tried"],
            "steps": steps}


def ctx_device(ctx) -> int:
    return 0

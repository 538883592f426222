"""Autotuner host logic (no GPU): candidate grid, cache keys, selection."""
import os

import pytest

from seismic_gb300 import autotune


def test_candidates_cover_both_kernels():
    c2 = autotune.candidates(True)
    assert any(c["step_kernel"] == 0 for c in c2)
    assert {c["tile_z"] for c in c2 if c["step_kernel"] == 1} == {32, 64, 128}
    c3 = autotune.candidates(False)
    assert {c["tile_y"] for c in c3 if c["step_kernel"] == 1} == {8, 16, 32, 64}


def test_select_picks_fastest_and_skips_failures():
    cands = [{"id": i} for i in range(5)]
    times = {0: 3.0, 1: 1.5, 2: None, 3: 2.0, 4: 1.6}

    def fn(c):
        t = times[c["id"]]
        if t is None:
            raise RuntimeError("rejected")
        return t

    best, res = autotune.select(cands, fn)
    assert best["id"] == 1
    assert sum(1 for r in res if r[2]) == 1


def test_select_raises_when_nothing_runs():
    with pytest.raises(RuntimeError):
        autotune.select([{"a": 1}], lambda c: (_ for _ in ()).throw(ValueError("x")))


def test_cache_roundtrip(tmp_path):
    p = os.path.join(tmp_path, "t.json")
    k = autotune.cache_key("GB300", 799, 1543, 1, 16)
    assert k == "GB300|832x1600x8|b16"
    autotune.save_cache({k: {"tuning": {"tile_z": 64}}}, p)
    assert autotune.load_cache(p)[k]["tuning"]["tile_z"] == 64
    assert autotune.load_cache(os.path.join(tmp_path, "missing.json")) == {}


def test_batch_candidates_cover_the_survey():
    assert autotune.batch_candidates(3) == [1, 2, 3]
    assert autotune.batch_candidates(16) == [1, 2, 4, 8, 16]
    assert autotune.batch_candidates(100) == [1, 2, 4, 8, 16, 32, 64]
    assert autotune.batch_candidates(1) == [1]


def test_select_batch_prefers_throughput_then_smaller():
    # Whole-sample seconds: launch overhead falls with batch size until the
    # device is full, then flattens.
    secs = {1: 8.0, 2: 4.1, 4: 2.2, 8: 1.5, 16: 1.5, 32: 1.7}
    b, res = autotune.select_batch(secs, lambda b: secs[b])
    assert b == 8
    assert len(res) == len(secs)

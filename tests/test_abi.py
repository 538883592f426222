"""The C-ABI library builds, loads without a GPU and exports every symbol
declared in include/swave.h; host-only entry points agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300.build import ROOT, build_library

HEADER = os.path.join(ROOT, "include", "swave.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sw_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    build_library()
    return sw.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n
    # and the Python mirror binds each of them with a signature
    assert set(names) <= set(sw._SIGS)


def test_version_and_no_device_error(lib):
    assert b"sm_103a" in lib.sw_version()
    h = C.c_void_p()
    code = lib.sw_ctx_create(10_000, C.byref(h))
    assert code in (sw.SW_BAD_PARAM, sw.SW_CUDA_ERR)


def test_vel_check_matches_oracle(lib, oracle):
    rng = np.random.default_rng(0)
    for twoD, dt, ok in ((True, 1e-3, True), (True, 2.5e-3, False), (False, 1e-3, True),
                         (False, 2.0e-3, False)):
        ny = 1 if twoD else 12
        g = sw.make_genpar(20, 30, ny, dz=10.0, dx=10.0, dy=10.0, dt=dt, twoD=twoD, fmax=30.0)
        v = rng.uniform(1500, 3000, (ny, 30, 20)).astype(np.float32)
        code, cour, sr = sw.vel_check(g, v)
        a, b = C.c_float(), C.c_float()
        vv = np.ascontiguousarray(v)
        ocode = oracle.load().oracle_vel_check(C.byref(g), vv.ctypes.data_as(C.POINTER(C.c_float)),
                                               C.byref(a), C.byref(b))
        assert code == ocode
        assert (code == sw.SW_OK) == ok
        assert cour == a.value and sr == b.value


def test_born_wavelet_matches_oracle(lib, oracle):
    from seismic_gb300 import synth
    w = synth.ricker(20.0, 5e-4, 500)
    a = sw.born_wavelet(w, 5e-4)
    b = w.copy()
    oracle.load().oracle_born_wavelet(b.ctypes.data_as(C.POINTER(C.c_float)), b.size, 5e-4)
    np.testing.assert_array_equal(a, b)
    assert a[0] == 0 and a[-1] == 0


def test_window_helpers_match_the_oracle_job_windowing(lib):
    """sw_shot_window / sw_window_extract / sw_window_scatter_add: the
    extract_coord_source_receiver_patch window, nearest-column extraction
    clamped to the model, and the in-model scatter-add (host only)."""
    g = sw.make_genpar(12, 50, 1, dz=10.0, dx=10.0, ox=100.0)
    rec = np.zeros((5, 3), np.float32)
    rec[:, 1] = [150.0, 200.0, 260.0, 300.0, 333.0]
    sou = np.array([5.0, 120.0, 0.0], np.float32)
    w, gw = sw.shot_window(g, 400.0, 0.0, sou, rec)
    # centre = midpoint range [135, 226.5] -> 180.75; window [-19.25, 380.75]
    assert w.oxw == np.float32(-19.25) and w.endx == np.float32(380.75)
    assert w.nxw == 41 and gw.nx == 41 and gw.ox == w.oxw
    big = np.arange(50 * 12, dtype=np.float32).reshape(50, 12)
    small = sw.window_extract(g, w, big)
    ix = np.clip(np.rint((w.oxw + 10.0 * np.arange(41) - 100.0) / 10.0).astype(int), 0, 49)
    np.testing.assert_array_equal(small, big[ix])
    acc = np.zeros_like(big)
    sw.window_scatter_add(g, w, np.ones_like(small), acc)
    inside = np.rint((w.oxw + 10.0 * np.arange(41) - 100.0) / 10.0).astype(int)
    inside = inside[(inside >= 0) & (inside < 50)]
    expect = np.zeros(50, np.float32)
    np.add.at(expect, inside, 1.0)
    np.testing.assert_array_equal(acc[:, 0], expect)


def test_rho_wavelet_matches_oracle_and_shifts_half_a_sample(lib, oracle):
    """sw_rho_wavelet (readsou withRho, ReadSouVelRho.f90:328-343): the
    same floats as the oracle; the result samples the wavelet half a step
    later, w'(t) = w(t + dt/2), so its energy centre moves half a sample
    earlier."""
    from seismic_gb300 import synth
    w = synth.ricker(15.0, 1e-3, 400).astype(np.float32)
    a = sw.rho_wavelet(w, 7)
    b = w.copy()
    oracle.load().oracle_rho_wavelet(b.ctypes.data_as(C.POINTER(C.c_float)), b.size, 7)
    np.testing.assert_array_equal(a, b)
    t = np.arange(400)
    peak = lambda x: np.sum(t * x ** 2) / np.sum(x ** 2)
    assert abs((peak(a) - peak(w)) + 0.5) < 0.02


def test_mute_mask_matches_oracle(lib, oracle):
    """sw_mute_mask (MuteParam_compute_mask, Mute.f90:50-95,172-219)."""
    nt, dt, ot = 600, 4e-3, 0.0
    sou = np.array([10.0, 1000.0, 0.0], np.float32)
    rec = np.zeros((40, 3), np.float32)
    rec[:, 1] = np.linspace(200.0, 2600.0, 40)
    args = (1500.0, 2500.0, 0.1, 1.6, 0.3)
    a = np.zeros((40, nt), np.float32)
    assert lib.sw_mute_mask(40, nt, C.c_float(dt), C.c_float(ot), sw.fptr(sou), sw.fptr(rec),
                            *[C.c_float(x) for x in args], sw.fptr(a)) == sw.SW_OK
    b = np.zeros_like(a)
    oracle.load().oracle_mute_mask(40, nt, dt, ot, sou.ctypes.data_as(C.POINTER(C.c_float)),
                                   rec.ctypes.data_as(C.POINTER(C.c_float)), *args,
                                   b.ctypes.data_as(C.POINTER(C.c_float)))
    np.testing.assert_array_equal(a, b)
    assert a.min() == 0.0 and a.max() == 1.0
    # the top mute moves later with offset
    first = [(np.argmax(row > 0.5)) for row in a]
    assert first[0] > first[20] and first[-1] > first[20]

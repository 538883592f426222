"""Pins of the oracle's band-pass (Bandpass.f90:89-149 with the Butterworth
filters of bandpass.c): pass band, stop band, zero phase, the refused
all-pass request."""
import numpy as np
import pytest

DT, NT = 2e-3, 2000


def _tone(f):
    t = np.arange(NT) * DT
    return np.sin(2 * np.pi * f * t).astype(np.float32)[None, :]


def _gain(oracle, f, **kw):
    x = _tone(f)
    y = oracle.bandpass(x, DT, **kw)
    mid = slice(400, 1600)
    return np.sqrt(np.mean(y[0, mid] ** 2) / np.mean(x[0, mid] ** 2))


def test_highcut_passes_low_and_stops_high_frequencies(oracle):
    assert abs(_gain(oracle, 5.0, fhi=20.0) - 1.0) < 0.01
    assert _gain(oracle, 60.0, fhi=20.0) < 1e-3
    # 14 poles, zero phase (7 each way): the gain at the cutoff is 1/2
    assert abs(_gain(oracle, 20.0, fhi=20.0) - 0.5) < 0.03


def test_lowcut_stops_low_frequencies(oracle):
    assert _gain(oracle, 1.0, flo=8.0, fhi=40.0) < 1e-3
    assert abs(_gain(oracle, 20.0, flo=8.0, fhi=40.0) - 1.0) < 0.01


def test_zero_phase_keeps_a_pulse_in_place(oracle):
    x = np.zeros((1, NT), np.float32)
    t = (np.arange(NT) - 1000) * DT
    x[0] = np.exp(-(t / 0.01) ** 2)
    y0 = oracle.bandpass(x, DT, fhi=30.0, phase=0)
    y1 = oracle.bandpass(x, DT, fhi=30.0, phase=1)
    assert abs(int(np.argmax(y0[0])) - 1000) <= 1
    assert int(np.argmax(y1[0])) > 1003          # minimum phase delays the pulse


def test_all_pass_request_is_refused(oracle):
    with pytest.raises(RuntimeError):
        oracle.bandpass(_tone(5.0), DT, flo=0.0, fhi=300.0)

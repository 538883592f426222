"""Seeded synthetic models, wavelets and acquisition geometries.

The reference's own workflows read field models (Marmousi, BP, Volve) that
are not available; these generators reproduce the shapes, spacings and
value ranges of the benchmark configurations instead:

* ``config1``: nz=201 x nx=401, 10 m, three flat layers 1500/2000/2500 m/s
  (interfaces at z=600 m and z=1300 m) with a +10 % Gaussian anomaly
  (sigma 150 m) at z=1000 m, x=2000 m; one 15 Hz Ricker at the surface
  centre; 401 receivers at depth index 2; 40-cell padding; dt=1 ms, 2000
  steps.
* ``layered_faulted``: dipping layers, normal faults with 20-80 m throw and
  3 % multiplicative correlated noise, clipped to [1500, 4700] m/s (the
  generator of the batched RTM, Born and FWI configurations).
* ``rtm_shots``: 37.5 m shot spacing, per-shot split-spread aperture of
  3-6 km and record length of 3-4 s.
* ``config2``: the batched-RTM survey, 751 x 2301 at 4 m, dt 0.375 ms (the
  scheme's Courant limit rules out 0.4 ms at 4700 m/s), 240 shots, 20 Hz
  Ricker, generator seed 2.
* ``config3``: the Born / FWI-gradient grid, 1201 x 3401 at 6.25 m, dt
  0.5 ms, background = the layered-faulted generator (seed 3) smoothed by a
  150 m Gaussian, reflectivity = 1 % density spikes N(0, 0.05) relative.
* ``config5``: the 3D survey, 200 (z) x 400 (x) x 400 (y) at 12.5 m, dt
  0.9 ms (the stated 1 ms exceeds the 3D Courant limit), 3 s; 25 dipping
  layers, 4 planar faults and a Gaussian salt body at 4500 m/s (seed 5);
  64 shots on an 8 x 8 surface grid, receivers every 100 m over the model.
"""
from __future__ import annotations

import math

import numpy as np


def ricker(f0: float, dt: float, nt: int, t0: float | None = None) -> np.ndarray:
    """Ricker wavelet (1 - 2 pi^2 f^2 tau^2) exp(-pi^2 f^2 tau^2), tau = t - t0."""
    if t0 is None:
        t0 = 1.5 / f0
    t = np.arange(nt, dtype=np.float64) * dt - t0
    a = (math.pi * f0 * t) ** 2
    return ((1.0 - 2.0 * a) * np.exp(-a)).astype(np.float32)


def config1_model() -> dict:
    nz, nx, d = 201, 401, 10.0
    z = np.arange(nz) * d
    x = np.arange(nx) * d
    Z, X = np.meshgrid(z, x, indexing="ij")
    v = np.where(Z < 600.0, 1500.0, np.where(Z < 1300.0, 2000.0, 2500.0))
    r2 = (Z - 1000.0) ** 2 + (X - 2000.0) ** 2
    v = v * (1.0 + 0.1 * np.exp(-r2 / (2 * 150.0 ** 2)))
    # Fortran order a(nz, nx): z fastest -> store as (nx, nz) C array.
    vel = np.ascontiguousarray(v.T, dtype=np.float32)
    return {"nz": nz, "nx": nx, "d": d, "vel": vel}


def config1(nt: int = 2000) -> dict:
    """Plain 2D modelling case (CPU-runnable) with the acquisition above."""
    from . import make_genpar
    m = config1_model()
    g = make_genpar(m["nz"], m["nx"], 1, dz=10.0, dx=10.0, dt=1e-3, nt=nt, ntaper=40,
                    lsinc=7, snapi=4, fmax=45.0)
    sou = np.array([0.0, 2000.0, 0.0], np.float32)
    rec = np.zeros((m["nx"], 3), np.float32)
    rec[:, 0] = 10.0            # Fortran z index 2
    rec[:, 1] = np.arange(m["nx"]) * 10.0
    w = ricker(15.0, 1e-3, nt, 0.1)
    return {"g": g, "vel": m["vel"], "sou": sou, "rec": rec, "wavelet": w}


def _smooth_noise(rng, shape, corr: float) -> np.ndarray:
    from scipy.ndimage import gaussian_filter
    n = rng.standard_normal(shape)
    n = gaussian_filter(n, sigma=corr, mode="reflect")
    return n / max(n.std(), 1e-12)


def layered_faulted(nz: int, nx: int, d: float, seed: int, nlayers: int = 40, nfaults: int = 6,
                    noise: float = 0.03, corr: float = 5.0, vmin: float = 1500.0,
                    vmax: float = 4700.0) -> np.ndarray:
    """Returns vel as a C array of shape (nx, nz) (Fortran a(nz, nx))."""
    rng = np.random.default_rng(seed)
    zmax, xmax = (nz - 1) * d, (nx - 1) * d
    z = np.arange(nz) * d
    x = np.arange(nx) * d
    Z, X = np.meshgrid(z, x, indexing="ij")
    Zeff = Z.copy()
    for _ in range(nfaults):
        xf = rng.uniform(0.1, 0.9) * xmax
        slope = math.tan(math.radians(rng.uniform(55.0, 70.0))) * rng.choice([-1.0, 1.0])
        throw = rng.uniform(20.0, 80.0)
        hanging = X > xf + Z / slope
        Zeff = np.where(hanging, Zeff - throw, Zeff)
    depths = np.sort(rng.uniform(0.03, 0.97, nlayers)) * zmax
    dips = rng.uniform(-0.1, 0.1, nlayers)
    xc = 0.5 * xmax
    idx = np.zeros((nz, nx), np.int32)
    for k in range(nlayers):
        idx += (Zeff > depths[k] + dips[k] * (X - xc)).astype(np.int32)
    base = vmin + (vmax - 300.0 - vmin) * (np.arange(nlayers + 1) / nlayers)
    jitter = rng.uniform(-120.0, 120.0, nlayers + 1)
    vl = np.clip(base + jitter, vmin, vmax)
    v = vl[idx]
    v = v * (1.0 + noise * _smooth_noise(rng, (nz, nx), corr))
    v = np.clip(v, vmin, vmax)
    return np.ascontiguousarray(v.T, dtype=np.float32)


def smooth(vel: np.ndarray, d: float, sigma_m: float) -> np.ndarray:
    from scipy.ndimage import gaussian_filter
    return np.ascontiguousarray(gaussian_filter(vel.astype(np.float64), sigma=sigma_m / d,
                                                mode="nearest"), dtype=np.float32)


def rtm_shots(nx: int, d: float, nshot: int, spacing: float, seed: int, dt: float,
              ap_range=(3000.0, 6000.0), rec_len=(3.0, 4.0), rec_step: int = 3,
              x0: float | None = None) -> list[dict]:
    """Surface shots with their own receiver spread and record length."""
    rng = np.random.default_rng(seed)
    xmax = (nx - 1) * d
    if x0 is None:
        x0 = 0.5 * (xmax - (nshot - 1) * spacing)
    shots = []
    for s in range(nshot):
        sx = x0 + s * spacing
        ap = rng.uniform(*ap_range)
        lo = max(0.0, sx - ap / 2)
        hi = min(xmax, sx + ap / 2)
        lo = math.floor(lo / d) * d
        hi = math.floor(hi / d) * d
        rx = np.arange(lo, hi + 0.5 * d, rec_step * d, dtype=np.float64)
        rec = np.zeros((rx.size, 3), np.float32)
        rec[:, 0] = d           # depth index 2
        rec[:, 1] = rx
        nt = int(round(rng.uniform(*rec_len) / dt))
        shots.append({"sou": np.array([0.0, sx, 0.0], np.float32), "rec": rec, "nt": nt,
                      "lo": lo, "hi": max(hi, rx[-1])})
    return shots


# Batched-RTM survey (751 x 2301 at 4 m).
CONFIG2 = {"nz": 751, "nx": 2301, "d": 4.0, "dt": 3.75e-4, "snapi": 4, "ntaper": 20,
           "f0": 20.0, "nshot": 240, "spacing": 37.5, "seed": 2}


def config2(nt_cap: int | None = None) -> tuple:
    """(genpar of the full model, vel (nx, nz), wavelet, shots): the 240-shot
    survey with per-shot apertures of 3-6 km and records of 3-4 s; genpar.nt
    is the longest record.  nt_cap truncates every record."""
    from . import make_genpar
    c = CONFIG2
    vel = layered_faulted(c["nz"], c["nx"], c["d"], seed=c["seed"])
    shots = rtm_shots(c["nx"], c["d"], c["nshot"], c["spacing"], seed=c["seed"], dt=c["dt"])
    if nt_cap:
        for s in shots:
            s["nt"] = min(s["nt"], nt_cap)
    ntmax = max(s["nt"] for s in shots)
    g = make_genpar(c["nz"], c["nx"], 1, dz=c["d"], dx=c["d"], dt=c["dt"], nt=ntmax,
                    ntaper=c["ntaper"], lsinc=7, snapi=c["snapi"], fmax=50.0)
    return g, vel, ricker(c["f0"], c["dt"], ntmax), shots


def config2_window(shot: dict) -> tuple[int, int]:
    """Columns [i0, i0 + nxw) of a config-2 shot's window with aperture 0:
    the patch spanned by the source and its receivers
    (extract_coord_source_receiver_patch, ExtractPadModel.f90:19-85).  The
    receivers of these shots bracket the source and sit on grid columns."""
    d = CONFIG2["d"]
    rx = np.asarray(shot["rec"])[:, 1]
    lo = min(float(rx.min()), float(shot["sou"][1]))
    hi = max(float(rx.max()), float(shot["sou"][1]))
    return int(round(lo / d)), int(round((hi - lo) / d)) + 1


# Born / FWI-gradient grid (1201 x 3401 at 6.25 m).
CONFIG3 = {"nz": 1201, "nx": 3401, "d": 6.25, "dt": 5e-4, "nt": 10000, "snapi": 4,
           "ntaper": 20, "f0": 15.0, "nshot": 120, "seed": 3}


def config3(nt: int | None = None, rec_step: int = 2) -> dict:
    """Smoothed background, sparse reflectivity and the 120 surface shots
    (full-width spread, a receiver every rec_step columns at depth index 2).
    Arrays are (nx, nz) C order = Fortran (nz, nx)."""
    from . import make_genpar
    c = CONFIG3
    nz, nx, d = c["nz"], c["nx"], c["d"]
    nt = nt or c["nt"]
    raw = layered_faulted(nz, nx, d, seed=c["seed"])
    vel = smooth(raw, d, 150.0)
    rng = np.random.default_rng(c["seed"])
    spikes = rng.random(vel.shape) < 0.01
    ref = np.where(spikes, rng.normal(0.0, 0.05, vel.shape), 0.0).astype(np.float32)
    g = make_genpar(nz, nx, 1, dz=d, dx=d, dt=c["dt"], nt=nt, ntaper=c["ntaper"], lsinc=7,
                    snapi=c["snapi"], fmax=30.0)
    xmax = (nx - 1) * d
    sx = np.linspace(0.05 * xmax, 0.95 * xmax, c["nshot"])
    rx = np.arange(0, nx, rec_step) * d
    rec = np.zeros((rx.size, 3), np.float32)
    rec[:, 0] = d
    rec[:, 1] = rx
    shots = [np.array([2 * d, x, 0.0], np.float32) for x in sx]
    return {"g": g, "vel": vel, "ref": ref, "rec": rec, "shots": shots,
            "wavelet": ricker(c["f0"], c["dt"], nt)}


def layered_faulted_3d(nz: int, nx: int, ny: int, d: float, seed: int, nlayers: int = 25,
                       nfaults: int = 4, vmin: float = 1500.0, vmax: float = 4700.0,
                       salt_v: float = 4500.0) -> np.ndarray:
    """Dipping layers (dips in x and y), planar normal faults with 20-80 m
    throw and a Gaussian salt body (the region where an anisotropic
    Gaussian exceeds 1/2) at salt_v.  Returns a C array (ny, nx, nz) =
    Fortran a(nz, nx, ny)."""
    rng = np.random.default_rng(seed)
    zmax, xmax, ymax = (nz - 1) * d, (nx - 1) * d, (ny - 1) * d
    Z, X, Y = np.meshgrid(np.arange(nz) * d, np.arange(nx) * d, np.arange(ny) * d,
                          indexing="ij")
    Zeff = Z.copy()
    for _ in range(nfaults):
        # A plane through (xf, yf) at the surface, dipping 55-70 degrees.
        xf, yf = rng.uniform(0.2, 0.8) * xmax, rng.uniform(0.2, 0.8) * ymax
        az = rng.uniform(0.0, math.pi)
        nxv, nyv = math.cos(az), math.sin(az)
        slope = math.tan(math.radians(rng.uniform(55.0, 70.0)))
        throw = rng.uniform(20.0, 80.0)
        hanging = (X - xf) * nxv + (Y - yf) * nyv > Z / slope
        Zeff = np.where(hanging, Zeff - throw, Zeff)
    depths = np.sort(rng.uniform(0.03, 0.97, nlayers)) * zmax
    dx_, dy_ = rng.uniform(-0.08, 0.08, nlayers), rng.uniform(-0.08, 0.08, nlayers)
    idx = np.zeros(Z.shape, np.int32)
    for k in range(nlayers):
        idx += (Zeff > depths[k] + dx_[k] * (X - 0.5 * xmax) + dy_[k] * (Y - 0.5 * ymax)).astype(
            np.int32)
    base = vmin + (vmax - 300.0 - vmin) * (np.arange(nlayers + 1) / nlayers)
    vl = np.clip(base + rng.uniform(-100.0, 100.0, nlayers + 1), vmin, vmax)
    v = vl[idx]
    cz, cx, cy = rng.uniform(0.45, 0.65) * zmax, rng.uniform(0.35, 0.65) * xmax, \
        rng.uniform(0.35, 0.65) * ymax
    sz, sx, sy = rng.uniform(0.10, 0.15) * zmax, rng.uniform(0.10, 0.18) * xmax, \
        rng.uniform(0.10, 0.18) * ymax
    g = np.exp(-0.5 * (((Z - cz) / sz) ** 2 + ((X - cx) / sx) ** 2 + ((Y - cy) / sy) ** 2))
    v = np.where(g > 0.5, salt_v, v)
    return np.ascontiguousarray(np.transpose(v, (2, 1, 0)), dtype=np.float32)


CONFIG5 = {"nz": 200, "nx": 400, "ny": 400, "d": 12.5, "dt": 9e-4, "t": 3.0, "snapi": 4,
           "ntaper": 20, "f0": 15.0, "seed": 5, "rec_step": 8}


def config5(nt: int | None = None) -> dict:
    """Model genpar, velocity (ny, nx, nz), wavelet, the 64 shots (sources
    on an 8 x 8 grid at 25 m depth) and the receiver patch every rec_step
    cells at 12.5 m depth (6 km x 6 km patches cover the 5 km model, so
    every shot records the whole grid)."""
    from . import make_genpar
    c = CONFIG5
    nz, nx, ny, d = c["nz"], c["nx"], c["ny"], c["d"]
    nt = nt or int(round(c["t"] / c["dt"]))
    vel = layered_faulted_3d(nz, nx, ny, d, seed=c["seed"])
    g = make_genpar(nz, nx, ny, dz=d, dx=d, dy=d, dt=c["dt"], nt=nt, ntaper=c["ntaper"],
                    lsinc=7, snapi=c["snapi"], twoD=False, fmax=30.0)
    st = c["rec_step"]
    rx, ry = np.meshgrid(np.arange(0, nx, st) * d, np.arange(0, ny, st) * d, indexing="ij")
    rec = np.zeros((rx.size, 3), np.float32)
    rec[:, 0], rec[:, 1], rec[:, 2] = d, rx.ravel(), ry.ravel()
    sx = np.linspace(0.1, 0.9, 8) * (nx - 1) * d
    sy = np.linspace(0.1, 0.9, 8) * (ny - 1) * d
    shots = [{"sou": np.array([2 * d, x, y], np.float32), "rec": rec, "nt": nt}
             for y in sy for x in sx]
    return {"g": g, "vel": vel, "wavelet": ricker(c["f0"], c["dt"], nt), "shots": shots}

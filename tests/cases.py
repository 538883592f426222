"""Small seeded cases shared by the parity tests (sizes the oracle finishes in seconds)."""
from __future__ import annotations

import numpy as np

import seismic_gb300 as sw
from seismic_gb300 import synth


def model2d(nz=60, nx=80, d=10.0, seed=0):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, :] * d
    x = np.arange(nx)[:, None] * d
    v = 1800.0 + 0.9 * z + 150.0 * np.sin(x / 170.0 + rng.uniform(0, 6)) + 40 * rng.standard_normal((nx, nz))
    return np.ascontiguousarray(v, np.float32)  # (nx, nz) = Fortran a(nz, nx)


def model3d(nz=30, nx=36, ny=32, d=10.0, seed=0):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, None, :] * d
    x = np.arange(nx)[None, :, None] * d
    y = np.arange(ny)[:, None, None] * d
    v = 1800.0 + 0.9 * z + 100.0 * np.sin(x / 150.0) * np.cos(y / 130.0) + 30 * rng.standard_normal((ny, nx, nz))
    return np.ascontiguousarray(v, np.float32)  # (ny, nx, nz) = Fortran a(nz, nx, ny)


def case2d(nz=60, nx=80, nt=300, ntaper=10, seed=0, dt=1.5e-3, nrec=None, f0=12.0, snapi=4):
    d = 10.0
    g = sw.make_genpar(nz, nx, 1, dz=d, dx=d, dt=dt, nt=nt, ntaper=ntaper, lsinc=7, snapi=snapi,
                       fmax=30.0)
    vel = model2d(nz, nx, d, seed)
    sou = np.array([20.0 + 0.37, (nx // 2) * d + 3.1, 0.0], np.float32)
    nrec = nrec or nx
    rec = np.zeros((nrec, 3), np.float32)
    rec[:, 0] = d + 2.3
    rec[:, 1] = np.linspace(0, (nx - 1) * d, nrec)
    w = synth.ricker(f0, dt, nt)
    return g, vel, sou, rec, w


def case3d(nz=30, nx=36, ny=32, nt=120, ntaper=8, seed=0, dt=1.5e-3, f0=12.0, snapi=4):
    d = 10.0
    g = sw.make_genpar(nz, nx, ny, dz=d, dx=d, dy=d, dt=dt, nt=nt, ntaper=ntaper, lsinc=7,
                       snapi=snapi, twoD=False, fmax=30.0)
    vel = model3d(nz, nx, ny, d, seed)
    sou = np.array([30.0 + 0.4, (nx // 2) * d + 2.0, (ny // 2) * d - 1.5], np.float32)
    rx, ry = np.meshgrid(np.arange(2, nx - 2, 3) * d, np.arange(2, ny - 2, 4) * d, indexing="ij")
    rec = np.zeros((rx.size, 3), np.float32)
    rec[:, 0] = d + 1.1
    rec[:, 1] = rx.ravel()
    rec[:, 2] = ry.ravel()
    w = synth.ricker(f0, dt, nt)
    return g, vel, sou, rec, w

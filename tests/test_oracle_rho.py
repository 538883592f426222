"""Pins of the oracle's variable-density operator (withRho:
FD_{2D,3D}_derivatives_acoustic_forward_grid, FDderivatives.f90:263-382,
588-657, with the half-cell sinc interpolation of Interpolate.f90:44-130)."""
import numpy as np
import pytest

import seismic_gb300 as sw


def _grid(g):
    n3p, n2p, n1p = sw.padded_shape(g)
    lo = -g.ntaper + 1 - 4
    z = (np.arange(n1p) + lo) * g.dz
    x = (np.arange(n2p) + lo) * g.dx
    y = (np.arange(n3p) + lo) * g.dy if not g.twoD else np.zeros(1)
    return np.meshgrid(y, x, z, indexing="ij")


@pytest.mark.parametrize("three_d", [False, True])
def test_rho_operator_is_exact_on_polynomials_with_unit_density(oracle, three_d):
    """With rho = 1 the staggered pair (gradient at half cells, divergence
    back) reproduces the Laplacian of polynomials up to rounding, away from
    the first-order padding cells."""
    if three_d:
        g = sw.make_genpar(24, 26, 22, dz=10.0, dx=12.0, dy=8.0, ntaper=6, twoD=False)
    else:
        g = sw.make_genpar(40, 44, 1, dz=10.0, dx=12.0, ntaper=6)
    Y, X, Z = _grid(g)
    shape = (g.ny, g.nx, g.nz) if three_d else (g.nx, g.nz)
    vel, rho = np.ones(shape), np.ones(shape)
    cases = [(Z ** 2, 2.0 + 0 * Z), (X ** 2, 2.0 + 0 * Z),
             (Z ** 4 / 1e4, 12 * Z ** 2 / 1e4),
             (Z ** 3 * X ** 3 / 1e9, (6 * Z * X ** 3 + 6 * X * Z ** 3) / 1e9)]
    if three_d:
        cases.append((Y ** 2 * Z ** 2 / 1e3, (2 * Z ** 2 + 2 * Y ** 2) / 1e3))
    m = 4 + 4 + 4
    sl = (slice(m, -m) if three_d else slice(None), slice(m, -m), slice(m, -m))
    for u, lap in cases:
        out = oracle.stencil_rho_f64(g, vel, rho, u)
        err = np.abs(out[sl] - lap[sl]).max() / np.abs(lap[sl]).max()
        assert err < 1e-12, err


def test_rho_operator_converges_for_smooth_density(oracle):
    """rho = exp(z/300), u = z^2: rho d/dz(u'/rho) = 2 - 2z/300 away from the
    model edges (where the padding replicates rho); the error falls by more
    than 8x when the spacing halves."""
    errs = []
    for dz in (10.0, 5.0):
        nz = int(600 / dz)
        g = sw.make_genpar(nz, 30, 1, dz=dz, dx=10.0, ntaper=6)
        Y, X, Z = _grid(g)
        zp = np.arange(1, nz + 1) * dz
        rho = np.repeat(np.exp(zp / 300.0)[None, :], g.nx, 0)
        out = oracle.stencil_rho_f64(g, np.ones_like(rho), rho, Z ** 2)[0]
        lo = -g.ntaper + 1 - 4
        sl = slice(-lo + 1 + 8, -lo + nz - 8)
        errs.append(np.abs(out[15, sl] - (2 - 2 * Z[0, 15, sl] / 300.0)).max())
    assert errs[0] < 1e-6 and errs[0] / errs[1] > 8.0, errs


def test_constant_density_scales_the_data(oracle):
    """Constant rho: the operator is rho-independent (rho2 = rho up to
    rounding) and the injection weight v^2*rho scales the data by rho.  The
    staggered operator differs from the constant-density Laplacian by
    discretisation only."""
    from tests.cases import case2d
    g, vel, sou, rec, w = case2d(nt=300)
    d = sw.SwPropDesc()
    d.g = g
    d.tmin, d.tmax, d.tstep = 1, g.nt, 1
    d.fd_scheme, d.injection, d.extraction = sw.FD_FORWARD, sw.INJ_SINC, sw.EXT_SINC
    out = {}
    for key, rho in (("one", np.ones_like(vel)), ("k", np.full_like(vel, 2.5)), ("none", None)):
        tr = np.zeros((rec.shape[0], g.nt), np.float32)
        oracle.propagate(d, vel, sou, w, rec, tr, rho=rho)
        out[key] = tr
    a, b = out["one"].astype(np.float64), out["k"].astype(np.float64)
    assert np.linalg.norm(b - 2.5 * a) / np.linalg.norm(b) < 2e-5
    rel = np.linalg.norm(a - out["none"]) / np.linalg.norm(out["none"])
    assert rel < 2e-3, rel     # 3.6e-4 measured


def _afwi_rho_run(oracle, g, vel, sou, w, rec, data, rho, imaging):
    n = vel.size
    wave = np.zeros((g.nt // g.snapi) * n, np.float32)
    d = sw.SwPropDesc()
    d.g, d.tmin, d.tmax, d.tstep = g, 1, g.nt, 1
    d.fd_scheme, d.injection, d.extract_wave = sw.FD_FORWARD, sw.INJ_SINC, 1
    oracle.propagate(d, vel, sou, w, wave=wave, rho=rho)
    b = sw.SwPropDesc()
    b.g, b.tmin, b.tmax, b.tstep = g, g.nt, 1, -1
    b.fd_scheme, b.injection, b.imaging = sw.FD_FORWARD, sw.INJ_SINC, imaging
    im, im2, il = (np.zeros(n, np.float32) for _ in range(3))
    oracle.propagate(b, vel, rec, data, wave=wave, image=im, illum=il, rho=rho,
                     image2=im2 if imaging == sw.IMG_AFWI_RHO else None)
    return im, im2, il


def test_afwi_rho_imaging_pins(oracle):
    """Imaging_condition_AFWI_RHOVP_from_memory (Imaging.f90:424-511): its
    illumination is the AFWI one; with a constant density c its velocity
    gradient is 2/c times the AFWI image (Imaging.f90:410-411) up to
    rounding; both gradients are linear in the receiver data.  The density
    2 makes the velocity gradient equal the AFWI image."""
    from tests.cases import case2d
    g, vel, sou, rec, w = case2d(nt=160)
    data = (np.random.default_rng(3).standard_normal((rec.shape[0], g.nt)) * 1e-2).astype(np.float32)
    rho = np.full(vel.shape, 2.0, np.float32)
    im, im2, il = _afwi_rho_run(oracle, g, vel, sou, w, rec, data, rho, sw.IMG_AFWI_RHO)
    ia, _, ila = _afwi_rho_run(oracle, g, vel, sou, w, rec, data, rho, sw.IMG_AFWI)
    np.testing.assert_array_equal(il, ila)
    assert np.abs(im).max() > 0 and np.abs(im2).max() > 0
    assert np.linalg.norm(im - ia) <= 1e-5 * np.linalg.norm(ia)
    im_2, im2_2, _ = _afwi_rho_run(oracle, g, vel, sou, w, rec, 2 * data, rho, sw.IMG_AFWI_RHO)
    # Exact up to subnormal intermediate values at the wavefront edges.
    assert np.abs(im_2 - 2 * im).max() <= 1e-6 * np.abs(im).max()
    assert np.abs(im2_2 - 2 * im2).max() <= 1e-6 * np.abs(im2).max()
    with pytest.raises(RuntimeError):
        _afwi_rho_run(oracle, g, vel, sou, w, rec, data, None, sw.IMG_AFWI_RHO)

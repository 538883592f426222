"""Pins of the oracle's free surface (surf_type, Boundary_set_free_surface_grid)
and mirror sources and receivers (shot_type, rec_type): two restatements of
a pressure-release surface at depth 0 agree, a mirror receiver doubles the
field of a mirrored source, and footprints outside the grid are refused."""
import numpy as np
import pytest

import seismic_gb300 as sw
from seismic_gb300 import synth


def _run(oracle, surf=0, shot=0, rec=0, depth=40.0, rz=30.0, oz=0.0, nt=500):
    g = sw.make_genpar(60, 100, 1, dz=10.0, dx=10.0, oz=oz, dt=1.5e-3, nt=nt, ntaper=10,
                       lsinc=7, snapi=4, fmax=30.0)
    g.surf_type, g.shot_type, g.rec_type = surf, shot, rec
    vel = np.full((100, 60), 2000.0, np.float32)
    sou = np.array([depth, 500.0, 0.0], np.float32)
    recs = np.zeros((50, 3), np.float32)
    recs[:, 0] = rz
    recs[:, 1] = np.linspace(50, 950, 50)
    d = sw.SwPropDesc()
    d.g = g
    d.tmin, d.tmax, d.tstep = 1, nt, 1
    d.fd_scheme, d.injection, d.extraction = sw.FD_FORWARD, sw.INJ_SINC, sw.EXT_SINC
    tr = np.zeros((50, nt), np.float32)
    oracle.propagate(d, vel, sou, synth.ricker(12.0, 1.5e-3, nt), recs, tr)
    return tr


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_free_surface_agrees_with_a_mirror_source(oracle):
    """A free surface on row 0 and a negated mirror source (with an absorbing
    top further up) both model the ghost of a shallow source: 3.3 % apart."""
    surf = _run(oracle, surf=1)
    mirror = _run(oracle, shot=1)
    none = _run(oracle)
    assert _rel(surf, mirror) < 0.06
    assert _rel(surf, none) > 0.3          # the ghost changes the data


def test_mirror_receiver_doubles_the_mirrored_field(oracle):
    """With a mirrored source the field is odd in depth, so a mirror receiver
    u(z) - u(-z) reads twice u(z): 5 % apart."""
    both = _run(oracle, shot=1, rec=1)
    src = _run(oracle, shot=1)
    assert _rel(both, 2 * src) < 0.08


def test_free_surface_between_rows_runs_the_sinc_mirror(oracle):
    """A surface 5 m below the model top (oz = -5 m) takes the sinc branch;
    the data stay close to the on-grid surface's."""
    a = _run(oracle, surf=1, oz=-5.0)
    b = _run(oracle, surf=1)
    assert np.isfinite(a).all() and 0.05 < _rel(a, b) < 0.3


def test_deep_mirror_source_is_refused(oracle):
    """The mirror of a source deeper than the extended top padding would land
    in the boundary cells: refused."""
    with pytest.raises(RuntimeError):
        _run(oracle, shot=1, depth=200.0)

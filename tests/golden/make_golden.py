"""Writes the golden fixtures (tests/golden/*.npz) from the FP32 oracle.

    python tests/golden/make_golden.py            # every case
    python tests/golden/make_golden.py rho_afwi2d # the named cases only

Each fixture holds a case's inputs and the oracle's outputs (arrays named
out_*).  The oracle's parity with the reference is unpinned (the Fortran
reference cannot be built here and ships no vectors for this path), so the
fixtures pin the oracle and the device path against regressions and across
machines, not against the reference itself."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import numpy as np  # noqa: E402

from oracle import bind  # noqa: E402
from seismic_gb300.build import build_oracle  # noqa: E402
from tests.golden.golden_cases import make_inputs, run  # noqa: E402


def main(names):
    build_oracle()
    cases = make_inputs()
    unknown = set(names) - set(cases)
    if unknown:
        raise SystemExit(f"unknown cases: {sorted(unknown)}")
    for name, inp in cases.items():
        if names and name not in names:
            continue
        out = run(bind, inp)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **inp, **out)
        print(f"{name}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main(sys.argv[1:])

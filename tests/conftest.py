import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libswave.so")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle import bind
    from seismic_gb300.build import build_oracle
    build_oracle()
    return bind


@pytest.fixture(scope="session")
def ctx():
    """A libswave context on cuda:0 (GPU tests only; fails loudly otherwise)."""
    if not _has_gpu():
        pytest.fail("GPU test collected on a machine without a visible CUDA device")
    from seismic_gb300.build import build_library
    build_library()
    import seismic_gb300 as sw
    c = sw.Context(0)
    yield c
    c.close()


def rel_l2(a, b) -> float:
    import numpy as np
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))

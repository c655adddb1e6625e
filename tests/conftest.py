import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libpixelflow_gb300.so")
    config.addinivalue_line("markers", "slow: long-running parity case")


def rel_l2(a, b):
    import numpy as np
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def rel_vel(got, ref, dim):
    """Relative L2 error of the velocity vector field (u, v[, w]) together."""
    import numpy as np
    keys = ("u", "v", "w")[:dim]
    num = sum(float(np.sum((np.asarray(got[k]) - np.asarray(ref[k])) ** 2)) for k in keys)
    den = sum(float(np.sum(np.asarray(ref[k]) ** 2)) for k in keys)
    return (num / max(den, 1e-300)) ** 0.5


@pytest.fixture
def rel():
    return rel_l2

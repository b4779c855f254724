import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: long CPU-side check")


def rms_rel(a, b):
    """sqrt(sum |a-b|^2 / sum |b|^2) over all particles and components."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def err_stats(a, b):
    """rms relative error (rms_rel) and the median and 99th percentile of the
    per-particle relative error |a_i - b_i| / |b_i| (particles with b_i = 0
    left out)."""
    a = np.asarray(a, dtype=np.float64).reshape(-1, 3)
    b = np.asarray(b, dtype=np.float64).reshape(-1, 3)
    nb = np.linalg.norm(b, axis=1)
    e = np.linalg.norm(a - b, axis=1)[nb > 0] / nb[nb > 0]
    return {"rms": rms_rel(a, b), "median": float(np.median(e)), "p99": float(np.percentile(e, 99))}


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.Port()

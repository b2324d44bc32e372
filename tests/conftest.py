import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "benchmark-euler-kernels_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for _p in (ROOT, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build(ref=False)
    return oracle


@pytest.fixture(scope="session")
def euler():
    """The CUDA library, built in-tree if missing (nvcc cross-compiles)."""
    import euler_gb300

    euler_gb300.build()
    euler_gb300.load()
    return euler_gb300


@pytest.fixture(scope="session")
def cuda(euler):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch


def rel_linf(a, b):
    """max|a-b| / max|b| per field (velocities start at exactly 0, so a
    pointwise relative error is not defined)."""
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = []
    for f in range(a.shape[0]):
        den = np.abs(b[f]).max()
        num = np.abs(a[f] - b[f]).max()
        out.append(num / den if den > 0 else num)
    return out

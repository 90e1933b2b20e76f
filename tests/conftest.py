import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libpps.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(ref=None)
    return O


@pytest.fixture(scope="session")
def pps_lib():
    import parallelpoissonsolver_gb300 as pps
    from parallelpoissonsolver_gb300 import build as B
    B.build()
    pps.load()
    return pps


@pytest.fixture(scope="session")
def gpu(pps_lib):
    if pps_lib.device_count() < 1:
        pytest.fail("GPU test run without a visible CUDA device")
    return pps_lib


def bits(a):
    return np.asarray(a, np.float64).view(np.uint64)


def same_bits(a, b) -> bool:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.shape != b.shape:
        return False
    # NaN payloads differ between x86 and the GPU; a NaN matches a NaN
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all((bits(a) == bits(b)) | both_nan))


def rel_l2(a, b) -> float:
    d = np.linalg.norm(np.asarray(a) - np.asarray(b))
    n = np.linalg.norm(np.asarray(b))
    return float(d / n) if n > 0 else float(d)


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))

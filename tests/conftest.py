import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsdd_gb300.so")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="session")
def built_lib():
    """Builds libsdd_gb300.so if needed (nvcc cross-compiles without a GPU) and returns its path."""
    from spectraldoublediffusiveconvection_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spectraldoublediffusiveconvection_gb300 import build
    build.build()
    return torch

import os
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libckgpu kernels)")


def load_golden(name: str):
    return np.load(GOLDEN / name)


@pytest.fixture(scope="session")
def golden():
    return load_golden


@pytest.fixture(scope="session")
def ck():
    """The libckgpu binding; GPU tests skip nothing: a missing GPU is a failure."""
    from clustkit_gb300 import _lib
    _lib.load()
    _lib.require_gpu()
    return _lib

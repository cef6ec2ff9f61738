"""Shared test setup: the `gpu` marker, import paths and fixture loaders."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    return load


@pytest.fixture(scope="session")
def engine():
    """The built engine; GPU tests fail loudly (no fallback) when it is missing."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected but no CUDA device is visible")
    from pydensecrf_gb300 import _lib
    _lib.load()
    from pydensecrf_gb300 import densecrf
    return densecrf

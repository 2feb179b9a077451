"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the built native library; the
rest run on CPU only (oracle vs golden vectors, host logic, C-ABI exports).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built native library")


@pytest.fixture(scope="session")
def golden_pairwise():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "reference_pairwise.npz")))


@pytest.fixture(params=["f32", "f64"])
def tag(request):
    return request.param

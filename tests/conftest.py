import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden_vectors():
    return np.load(os.path.join(GOLDEN, "reference_vectors.npz"))


@pytest.fixture(scope="session")
def golden_frames():
    return np.load(os.path.join(GOLDEN, "reference_frames.npz"))


@pytest.fixture(scope="session")
def golden_single():
    return np.load(os.path.join(GOLDEN, "reference_single.npz"))


@pytest.fixture(scope="session")
def golden_two_medium():
    return np.load(os.path.join(GOLDEN, "reference_two_medium.npz"))


@pytest.fixture(scope="session")
def cuda():
    """The GPU tests' device. On a machine with a GPU the native library must
    build and load (no fallback); without one the test is an error, not a skip."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from us_lab4a_gb300 import build, native
    build.build()
    native.load()
    return torch.device("cuda:0")

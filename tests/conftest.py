import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: runs the sm_103a CUDA kernels (needs a GB300)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.get(False)


@pytest.fixture(scope="session")
def orc64():
    import oracle
    return oracle.get(True)


@pytest.fixture(scope="session")
def gpu():
    """The default flof context on cuda:0; fails (never skips) when the
    library or the device is missing."""
    import ofblend_gb300 as F
    return F.context()


def rng(seed=0):
    return np.random.default_rng(seed)

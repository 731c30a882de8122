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
    # the native library and the oracle are built in-tree before any test imports them
    from gauxc_gb300 import build as _b
    _b.build()
    import oracle
    oracle.build()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def g():
    import gauxc_gb300
    return gauxc_gb300


@pytest.fixture(scope="session")
def has_gpu():
    import gauxc_gb300
    return gauxc_gb300.device_count() > 0

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def built_lib():
    """libpalgpu.so, built in-tree if missing (host compile only)."""
    from palinstrophy_gb300 import _lib
    from palinstrophy_gb300.build import build
    build(verbose=False)  # incremental: recompiles only stale units
    return _lib.load()

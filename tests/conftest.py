import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA core through the C ABI)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def rtlib():
    """The CUDA core's C ABI (built in-tree if missing)."""
    from raptor_gb300 import build, core
    if not os.path.exists(build.LIB):
        build.build()
    core.lib()
    return core


@pytest.fixture(scope="session")
def ctx(rtlib):
    c = rtlib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden_npz():
    import numpy as np
    return np.load(os.path.join(GOLDEN, "ref_small.npz"))

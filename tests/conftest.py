import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def goldens():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_goldens.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def lfg():
    """The GPU library (C-ABI through ctypes); built on first use."""
    import lehrfempp_gb300 as L
    L.load()
    return L


@pytest.fixture(scope="session")
def ctx(lfg):
    c = lfg.Context(0)
    yield c
    c.close()

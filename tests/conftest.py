import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and runs the CUDA kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    import __graft_entry__

    __graft_entry__.build()
    yield


@pytest.fixture(scope="session")
def gpu():
    import omnioperator_gb300 as omg

    if not omg.device_available():
        pytest.fail("GPU test run without a visible CUDA device")
    return omg

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libnlmgpu kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library; on a GPU machine a missing build is an error."""
    from nlmech_gb300 import build, gpu as g
    build.build()
    g.load()
    if g.device_count() < 1:
        pytest.fail("no CUDA device visible to libnlmgpu")
    return g

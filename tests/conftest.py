import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def pytest_sessionstart(session):
    # Build libvpt and the oracle once per session (incremental, seconds).
    import __graft_entry__
    __graft_entry__.build()


@pytest.fixture(scope="session")
def vpt():
    import voxelpathtracer_gb300 as v
    return v


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    return o


@pytest.fixture(scope="session")
def gpu(vpt):
    if not vpt.device_available():
        pytest.fail("a gpu-marked test ran without a usable CUDA device")
    return True

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs on the GPU box")


@pytest.fixture(scope="session")
def ctx():
    from bubblephysics_gb300 import _native as N
    from bubblephysics_gb300.solver import Context
    status = N.library().bp_device_available(0)
    if status != N.OK:
        pytest.fail("GPU test without a usable CUDA device: " + N.STATUS_NAMES[status])
    return Context(0)

TESTS = Path(__file__).resolve().parent
if str(TESTS) not in sys.path:
    sys.path.insert(0, str(TESTS))

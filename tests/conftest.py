import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a) and libsimgb.so")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def ctx():
    from simbuca_gb300.api import Context
    c = Context(0)
    yield c
    c.close()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and librheogpu.so")
    config.addinivalue_line("markers", "slow: long-running oracle cases")


@pytest.fixture(scope="session")
def ctx():
    from rheotool_gb300.runtime import Context
    c = Context(0)
    yield c
    c.close()

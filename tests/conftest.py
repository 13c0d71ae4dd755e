import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def engine_lib():
    from tfm_gb300 import build

    build.build()
    from tfm_gb300 import ccpgpu

    return ccpgpu.load()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build()
    oracle.lib()
    return oracle

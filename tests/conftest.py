import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def native_lib():
    from exadem_gb300 import build

    build.build()
    from exadem_gb300 import _abi

    return _abi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle

    return oracle.load()

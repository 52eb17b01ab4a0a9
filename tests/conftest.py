import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libwoogpu.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build
    build.build()
    from oracle import oracle
    return oracle.lib()


@pytest.fixture(scope="session")
def gpu_lib():
    from woodem_gb300 import _build, _native
    _build.build()
    return _native.lib()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmsl_gb300.so")


@pytest.fixture(scope="session")
def gpu():
    """Bind libmsl_gb300.so to cuda:0 (builds the library first if needed)."""
    from muesli4_gb300 import abi, build
    build.build()
    abi.init(0)
    yield abi
    abi.sync()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def orc():
    from oracle import binding
    binding.lib()
    return binding


@pytest.fixture(scope="session")
def vtlib():
    from voxeltoy_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def ctx():
    from voxeltoy_gb300 import Context
    c = Context()
    yield c
    c.close()

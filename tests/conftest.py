import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs through the CUDA C-ABI)")


@pytest.fixture(scope="session")
def native():
    """The built native library (built here if missing; compiling needs no GPU)."""
    from suzerain_gb300 import _native, build
    build.build()
    return _native.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O

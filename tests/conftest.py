import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    """The product library, built in-tree if missing (nvcc cross-compiles)."""
    from thesis_gb300 import build, native
    build.build()
    return native.lib()


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build_oracle()
    return pyoracle

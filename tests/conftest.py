import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def axbc():
    """The CUDA library, built in-tree if needed; fails loudly when missing."""
    from axbc_gb300 import build
    build.build()
    import axbc_gb300
    axbc_gb300.lib()
    return axbc_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")
    config.addinivalue_line("markers", "slow: longer-running case")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    return oracle.load()


@pytest.fixture(scope="session")
def plume_lib():
    """The product library, built in-tree (fails loudly when it cannot be built)."""
    from cfs_plume_gb300 import build, plume
    build.build()
    return plume.load_library()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    return g.package()


@pytest.fixture(scope="session")
def built_pkg():
    """Package with libshmsem.so and the oracle built (nvcc works without a GPU)."""
    import __graft_entry__ as g
    g.build()
    return g.package()

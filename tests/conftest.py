import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (the parity tests of the CUDA path)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def hyp():
    """The product package with its CUDA library built (raises if it cannot be)."""
    import hyperelasticsolver_gb300 as h
    h.build_library()
    h._lib.load()
    return h

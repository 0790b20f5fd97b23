import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle():
    import oracle as _oracle
    _oracle.build()
    return _oracle


@pytest.fixture(scope="session")
def gn():
    """The GPU library (built in-tree if needed)."""
    from pynear_gb300 import build as _build
    _build.build()
    import pynear_gb300
    return pynear_gb300


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))

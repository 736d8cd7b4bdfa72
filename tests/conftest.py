import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REFERENCE = "/root/reference"  # present only in the development container


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the device kernels")
    config.addinivalue_line("markers", "slow: large sizes")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def stocha():
    """The product package, built in-tree (nvcc cross-compiles without a GPU)."""
    from stocha_gb300 import build

    build.build()
    import stocha_gb300

    return stocha_gb300


@pytest.fixture(scope="session")
def reference_root():
    if not os.path.exists(os.path.join(REFERENCE, "src")):
        pytest.skip("reference tree not mounted here")
    return REFERENCE

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The reference source tree (heki1224/stocha), for the tests that read its
# tables as text; set STOCHA_REFERENCE_ROOT to its checkout.  Without it those
# tests skip and the committed fixtures carry the pins.
REFERENCE = os.environ.get("STOCHA_REFERENCE_ROOT", "")


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
    if not REFERENCE or not os.path.exists(os.path.join(REFERENCE, "src")):
        pytest.skip("reference tree not available (set STOCHA_REFERENCE_ROOT)")
    return REFERENCE

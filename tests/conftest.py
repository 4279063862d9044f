import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: larger parity cases")


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library; GPU tests fail loudly when it is missing."""
    from cassia_gb300 import abi
    return abi.load_library()

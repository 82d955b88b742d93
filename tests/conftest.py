import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: longer CPU checks")


@pytest.fixture(scope="session")
def built_lib():
    """Path of libsei_gb300.so, building it in-tree when missing (nvcc cross-compiles without a GPU)."""
    from seissol_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    return b.LIB

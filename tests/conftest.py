import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree; fails loudly when no GPU is usable."""
    from branson_gb300 import _lib
    return _lib.load()

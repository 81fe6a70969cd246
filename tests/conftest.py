import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running statistical check")


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library; fails loudly when it is missing on a GPU machine."""
    from opendust_gb300 import _build, _lib

    _build.build()
    lib = _lib.load()
    assert lib.od_device_count() > 0, "no CUDA device visible"
    return lib

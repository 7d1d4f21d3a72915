import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libember_gpu.so")
    config.addinivalue_line("markers", "slow: larger CPU oracle runs")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library, loaded; fails loudly when it cannot be used."""
    from ember_gb300 import _lib
    lib = _lib.lib()
    if lib.ember_device_count() < 1:
        pytest.fail("no CUDA device visible to libember_gpu.so")
    return lib

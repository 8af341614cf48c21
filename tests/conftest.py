import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than ~20 s on one CPU core")


@pytest.fixture(scope="session")
def csem_lib():
    import demo_matrixfree_csem_gb300 as cs
    return cs.lib()


@pytest.fixture(scope="session")
def gpu(csem_lib):
    import demo_matrixfree_csem_gb300 as cs
    if cs.device_count() < 1:
        pytest.fail("GPU test selected but no CUDA device is visible")
    return True

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103)")


@pytest.fixture(scope="session")
def gpu_ready():
    """Build libskidgpu if needed and check a device is present."""
    from skid_gb300 import build, gpu
    build.build_lib()
    gpu.load()
    return True

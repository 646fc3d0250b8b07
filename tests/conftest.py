import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds liblfm_gpu.so and the oracle port once per session (no-op when
    they are up to date)."""
    from lfm_public_gb300 import build
    build.build_library()
    build.build_port()
    yield

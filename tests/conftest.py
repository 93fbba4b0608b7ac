import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the native library")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native library and the C oracle once per session (cheap when
    up to date; nvcc cross-compiles without a GPU)."""
    from sayakaamr_gb300 import build
    build.build_library()
    build.build_oracle()
    yield

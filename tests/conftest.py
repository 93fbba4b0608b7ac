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


@pytest.fixture(autouse=True)
def _no_pending_cuda_error(request):
    """after every GPU test (its handles collected), the library leaves no
    CUDA runtime error pending: an error left behind would surface in an
    unrelated later call"""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    import gc
    import sayakaamr_gb300 as sg
    gc.collect()
    assert sg.cuda_peek_error() == 0, "CUDA error left pending: %d" % sg.cuda_peek_error()

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    lib = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
    if not os.path.exists(lib):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True,
                       capture_output=True)
    so = os.path.join(ROOT, "qll_gb300", "libqll_gb300.so")
    if not os.path.exists(so):
        from qll_gb300 import build
        build.build()


_ensure_built()


@pytest.fixture(autouse=True)
def _clear_library_error():
    """qllg_last_error() keeps the last message until the next error; start
    every test from a clean slate so a test sees only its own errors"""
    from qll_gb300 import qll
    qll.load().qllg_clear_error()
    yield

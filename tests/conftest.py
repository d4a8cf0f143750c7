import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from em_lab_gb300 import _build

    _build.build_oracle()
    try:
        _build.build_library()
    except RuntimeError:
        pass  # CPU-only checks that need the library skip themselves
    yield

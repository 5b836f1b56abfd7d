import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")
    config.addinivalue_line("markers", "reference: needs the reference checkout (skipped when absent)")


@pytest.fixture(scope="session")
def gpu_ctx():
    from pyzkp_gb300 import _native

    return _native.default_context()

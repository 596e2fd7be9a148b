import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE = os.path.join(ROOT, "oracle")
if ORACLE not in sys.path:
    sys.path.insert(0, ORACLE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


@pytest.fixture(scope="session")
def engine():
    """Builds (if stale) and loads the engine libraries; a GPU test fails if
    they cannot be built or loaded -- there is no CPU fallback."""
    from dsim_gb300 import build
    build.build()
    from dsim_gb300 import _lib
    _lib.native()
    return _lib

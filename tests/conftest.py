import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def gpu_context():
    """A library context on cuda:0; the CUDA library must be built and load."""
    from smuthi_gb300 import _lib
    from smuthi_gb300.build import build
    build()
    ctx = _lib.Context(0)
    yield ctx
    ctx.close()

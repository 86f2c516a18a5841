import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")


@pytest.fixture(scope="session")
def gpu_ctx():
    from trax_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()

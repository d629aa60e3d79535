import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built libcrt.so")


@pytest.fixture(scope="session")
def ctx():
    """One libcrt context for the GPU tests (fails loudly if the library or the GPU is missing)."""
    from realtimeraytracing_gb300 import crt
    c = crt.Context()
    yield c
    c.close()

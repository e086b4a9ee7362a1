"""pytest configuration: the `gpu` marker selects tests that need a GB300."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def ctx():
    import mymoonmd_gb300 as m
    c = m.Context(0)
    yield c
    c.close()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and the built libwtb_gb300.so")


@pytest.fixture(scope="session")
def built():
    """Builds the library and the oracle's C restatement once per session."""
    import __graft_entry__ as g

    g.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    from wtb_gb300 import api

    c = api.Context(0)
    yield c
    c.close()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    import __graft_entry__ as g
    g.build()
    import idp_gb300
    return idp_gb300.load()


@pytest.fixture(autouse=True)
def reference_call_defaults():
    """Every test starts the reference-shaped entry points from their
    defaults (precision mode, extra context parameters)."""
    from idp_gb300 import api

    mode, params = api.DiscreteShell.mode, dict(api.DiscreteShell.params)
    yield
    api.DiscreteShell.mode, api.DiscreteShell.params = mode, params

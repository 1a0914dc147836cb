import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tesina-rt_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (and the reference kernels where available) once."""
    import build as ob
    ob.build_oracle()
    ob.build_ref()
    yield


@pytest.fixture(scope="session")
def orc():
    import pyoracle
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def ctx():
    from rtgb import build as rb
    from rtgb import capi
    rb.build()
    c = capi.Context(0)
    yield c
    c.close()

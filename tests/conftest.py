"""Shared fixtures.  `-m gpu` tests need a CUDA device (libtcym.so); the rest
run on any host: the oracle against the reference's golden vectors, and the
device arithmetic through the test-only host build of the per-site code."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels through the C ABI)")


@pytest.fixture(scope="session")
def oracle_port():
    import oracle
    oracle.build()
    return {2: oracle.Port(2), 3: oracle.Port(3)}


@pytest.fixture(scope="session")
def hostcheck():
    from tests import _hostcheck
    return _hostcheck.load()


@pytest.fixture(scope="session")
def ctx():
    import topologicalcymsolver_gb300 as tcym
    c = tcym.Context(0)
    yield c
    c.close()

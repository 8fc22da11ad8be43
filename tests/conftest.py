"""Shared fixtures. GPU tests carry @pytest.mark.gpu and call the CUDA path
through the C ABI (libclbellard.so); CPU tests cover the oracle, the host
logic and the library's exports."""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cbl():
    import clbellard_gb300 as C
    C.load()
    return C


@pytest.fixture(scope="session")
def ctx192(cbl):
    c = cbl.Context(0, 1)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ctx_beta(cbl):
    c = cbl.Context(0, 2)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ctxdd(cbl):
    c = cbl.Context(0, 0)
    yield c
    c.close()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def z0p():
    import z0p_gb300

    z0p_gb300.build.build()
    return z0p_gb300


@pytest.fixture(scope="session")
def gpu_ctx(z0p):
    return z0p.default_context(0)

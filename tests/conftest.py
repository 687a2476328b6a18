import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmyqc.so")


def golden(*p):
    return os.path.join(GOLDEN, *p)


@pytest.fixture(scope="session")
def ftab():
    import oracle
    return oracle.read_ftab(golden("Ftab"))


@pytest.fixture(scope="session")
def basis_text():
    return open(golden("mybasis")).read()


@pytest.fixture(scope="session")
def ctx():
    from myqc_gb300.session import Context
    c = Context(0)
    yield c
    c.close()

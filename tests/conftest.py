import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def lib():
    """The built CUDA library (built on first use)."""
    from gpusharesat_gb300 import build
    build.build()
    import gpusharesat_gb300
    return gpusharesat_gb300.load()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def engine(lib):
    import gpusharesat_gb300 as g
    eng = g.Engine(0)
    yield eng
    eng.close()

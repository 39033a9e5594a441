import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from slothdb_gb300 import build
    build.build_oracle()
    import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def gblib():
    """The CUDA library, built in-tree if needed (no fallback)."""
    from slothdb_gb300 import build, capi
    build.build_lib()
    return capi.load()

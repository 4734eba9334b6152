import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def orc():
    return __graft_entry__.load_oracle()


@pytest.fixture(scope="session")
def ir():
    import gcchem.mechanism

    return gcchem.mechanism.load_ir()


@pytest.fixture(scope="session")
def solver():
    import gcchem.capi as capi

    s = capi.Solver(0)
    yield s
    s.close()

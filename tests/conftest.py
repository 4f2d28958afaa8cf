import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lri():
    """The package (host API + CUDA library), built in-tree on first use."""
    import __graft_entry__ as ge

    ge.load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def oracle():
    from oracle import lri_oracle

    return lri_oracle

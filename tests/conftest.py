import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "idealizedspectralgcm.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a) and the built libjgcm.so")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def jg(built):
    import jgcm

    return jgcm


@pytest.fixture(scope="session")
def orc(built):
    import oracle

    return oracle

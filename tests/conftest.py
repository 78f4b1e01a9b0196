import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "gvdb-voxels_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgvx.so")


@pytest.fixture(scope="session")
def gvx_mod():
    import gvx

    gvx.load()
    return gvx


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.load()
    return oracle

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libexposurerender.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib as OL
    return OL.load_oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle_lib as OL
    r = OL.load_ref()
    if r is None:
        pytest.skip("reference host build (oracle/_ref/liberref.so) not present on this machine")
    return r

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def gaia_lib():
    from gaia_gb300 import build as gb

    gb.build()
    import gaia_gb300

    return gaia_gb300

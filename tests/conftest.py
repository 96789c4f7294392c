import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def hs():
    import heterosync_gb300 as hs_mod
    hs_mod.lib()  # fail loudly if the library is missing
    return hs_mod


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.lib()
    return o

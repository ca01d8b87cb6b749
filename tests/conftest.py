import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_built():
    from oracle import build_oracle
    return build_oracle.build()


@pytest.fixture(scope="session")
def native_lib():
    import pandemicthrust_gb300 as pt
    pt.build()
    return pt.load_library()

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Compile the engine (nvcc, sm_103a) and the oracle once per session."""
    from pentrack_gb300 import build
    build.build_engine()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def oracle_mod(built):
    from oracle import pyoracle
    return pyoracle

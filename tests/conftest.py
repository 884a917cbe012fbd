import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libbfm.so")
    config.addinivalue_line("markers", "slow: large problem sizes")


@pytest.fixture(scope="session")
def libbfm_path():
    from bfm_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def libbfm(libbfm_path):
    import bfm_gb300
    return bfm_gb300.lib()

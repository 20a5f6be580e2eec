import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libgpe.so")


@pytest.fixture(scope="session")
def gpe():
    """The package (host mirror + ctypes binding) as module gpe_gb300."""
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def oracle():
    from oracle import gpe_oracle
    return gpe_oracle


@pytest.fixture(scope="session")
def lib(gpe):
    """libgpe.so, built on first use."""
    gpe.build()
    return gpe.load_library()

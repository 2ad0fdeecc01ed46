import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device; runs the compositor through the C ABI")


@pytest.fixture(scope="session")
def pkg():
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def hdsr_lib(pkg):
    """libhdsr.so, built for sm_103a if it is missing or stale."""
    pkg._build.build()
    return pkg.load_library()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def cuda(hdsr_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch

"""Test configuration.

Tests marked ``gpu`` need a CUDA device and call the product through its C ABI
(libtvk.so); everything else runs on the CPU: the oracle against the
reference's golden vectors and the reference's own converter, the host logic,
and the loading/exports of the C-ABI library.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from tuvok_gb300 import build
    build.build_all()
    try:
        build.build_reference()
    except RuntimeError:
        pass  # the reference's sources are only present where they were mounted
    yield


@pytest.fixture(scope="session")
def cuda_ok():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True

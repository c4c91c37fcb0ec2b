import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def native_lib():
    """Builds libsmartinterp.so if needed and returns the ctypes handle."""
    from biomedisa_gb300 import _native, build

    build.build()
    return _native.lib()


@pytest.fixture(scope="session")
def c_oracle():
    import oracle

    return oracle.c_oracle()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda", 0)

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300, sm_103a); runs the native library")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / f"{name}.npz")
    return load


@pytest.fixture(scope="session")
def built_lib():
    """The C-ABI library, built from source if it is not there yet."""
    from brisc_gb300 import build as B
    if not B.LIB.exists():
        B.build()
    return B.LIB


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from brisc_gb300 import build as B
    if not B.LIB.exists():
        B.build()
    torch.cuda.init()
    return torch.device("cuda:0")

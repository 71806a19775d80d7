import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built extension")


@pytest.fixture(scope="session")
def cuda_device():
    """Builds the extension if needed and checks that a GPU is visible."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a visible CUDA device")
    from rtc8_gb300 import build as b

    b.build()
    torch.cuda.init()
    return torch.device("cuda:0")

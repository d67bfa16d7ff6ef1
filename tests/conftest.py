import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


@pytest.fixture(scope="session")
def cuda_device():
    """The GPU tests run the CUDA kernels for real; without a device they fail."""
    import torch
    assert torch.cuda.is_available(), "GPU test collected on a machine without CUDA"
    return 0

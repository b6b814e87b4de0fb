import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libgpucsl_gb300.so")
    config.addinivalue_line("markers", "slow: longer CPU-side oracle runs")


@pytest.fixture(scope="session")
def cuda():
    """torch with a CUDA device, the library built and loaded."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from gpucsl_gb300 import build as gbuild
    gbuild.build()
    from gpucsl_gb300 import _lib
    _lib.lib()
    return torch

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfire.so")


@pytest.fixture(scope="session")
def cuda_lib():
    """Builds (if stale) and loads libfire.so; the product path has no CPU fallback."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    from sparse_wf_gb300.build import build
    from sparse_wf_gb300 import _lib

    build()
    return _lib.load()

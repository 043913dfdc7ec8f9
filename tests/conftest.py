import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libibm_rk3.so")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; fails loudly if absent."""
    if not _have_gpu():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    from interparts_mpich_gb300 import build as b
    b.build()
    from interparts_mpich_gb300.solver import load_library
    return load_library()

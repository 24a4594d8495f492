"""Shared fixtures.  `-m gpu` tests need a CUDA GPU; everything else runs on the CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a, GB300)")


@pytest.fixture(scope="session")
def nlod_lib():
    """Builds (incrementally) and loads libnlod.so."""
    from neural_lod_gb300.build import build_library
    from neural_lod_gb300._lib import load

    build_library()
    return load()


@pytest.fixture(scope="session")
def cuda():
    import torch

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    return torch.device("cuda:0")

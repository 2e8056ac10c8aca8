import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "g-mm-repair_gb300"))
sys.path.insert(0, str(REPO))
os.environ.setdefault("GMR_ENERGY", "0")  # legacy entry points: skip the 1.5 s NVML energy loop in tests


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the libgmr.so kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from gmr import build as gbuild
    from oracle import oracle
    gbuild.build()
    oracle.build()
    yield


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False

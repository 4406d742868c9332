import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the native library")


@pytest.fixture(scope="session", autouse=True)
def _native_library():
    """Build the in-tree native library once per session (fast no-op when up to date)."""
    from xped_gb300 import build as b
    b.build()
    yield


def gpu_available() -> bool:
    try:
        import torch  # noqa: F401
        return torch.cuda.is_available()
    except Exception:
        return os.path.exists("/dev/nvidia0")

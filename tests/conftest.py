import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libfrico_gpu.so; fails loudly if that is impossible."""
    import frico_gb300
    frico_gb300.build()
    from frico_gb300 import _abi
    return _abi.load()

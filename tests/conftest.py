import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib_built():
    """Build liboh_gb300.so if needed (CPU-only nvcc cross-compile is fine)."""
    from openholo_gb300 import build
    build.build()
    import openholo_gb300
    return openholo_gb300.lib()


@pytest.fixture(scope="session")
def ctx(lib_built):
    if not _cuda_ok():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from openholo_gb300 import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def dev():
    import torch
    return torch.device("cuda:0")

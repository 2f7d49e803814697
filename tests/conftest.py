import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the librq.so kernels)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds librq.so and the oracle library once per session (incremental)."""
    from candela_gb300 import _build
    from oracle import oracle as O

    _build.build()
    O.build()
    yield


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from candela_gb300 import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def nthreads():
    return os.cpu_count() or 1

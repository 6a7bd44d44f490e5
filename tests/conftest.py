import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def tc():
    """The engine package with its library built (GPU tests only)."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    import tensorcircuit_gb300 as tcg

    tcg.build()
    return tcg

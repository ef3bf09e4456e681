import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def oracle_mod():
    import pyoracle

    pyoracle.build()
    return pyoracle


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def swaplib():
    """The sm_103a library; GPU tests fail (not skip) if it cannot load."""
    from swap_gb300 import abi

    return abi.load()


def relerr(a, b):
    """max|a-b| / max|b| (0 when both are 0)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if a.size else 0.0
    return 0.0 if num == 0 else num / (den if den > 0 else 1.0)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    d = np.linalg.norm(a - b)
    n = np.linalg.norm(b)
    return 0.0 if d == 0 else d / (n if n > 0 else 1.0)

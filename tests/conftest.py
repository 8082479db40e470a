import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsbpmg.so")
    config.addinivalue_line("markers", "slow: large sizes")


@pytest.fixture(scope="session")
def golden():
    return np.load(ROOT / "tests" / "golden" / "sbp_golden.npz")


@pytest.fixture(scope="session")
def sbp():
    """The package with its CUDA library loaded (fails loudly if missing)."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import sc_2022_gb300 as m
    m.load_library()
    return m

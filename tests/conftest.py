import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103a) device and the built libpvd_gb300.so")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(GOLDEN / "reference_golden.npz")

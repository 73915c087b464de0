import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built librtr.so")


@pytest.fixture(scope="session")
def rtr():
    import realtime_robot_gb300 as R
    R.lib()  # fails loudly when the CUDA library has not been built
    return R


@pytest.fixture(scope="session")
def ctx(rtr):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected but no CUDA device is visible")
    c = rtr.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(ROOT / "tests" / "golden" / "pcd_pairs.npz")

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built CUDA library")


def track(name):
    import numpy as np

    return np.load(ROOT / "warporacer3d_gb300" / "tracks" / f"{name}.npz")["track"]


@pytest.fixture(scope="session")
def flat():
    return track("flat")


@pytest.fixture(scope="session")
def bridge():
    return track("bridge")


@pytest.fixture(scope="session")
def ramp():
    return track("ramp")


@pytest.fixture(scope="session")
def bank():
    return track("bank")

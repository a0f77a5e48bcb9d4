import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return GOLDEN


@pytest.fixture(scope="session")
def trajectories():
    return json.loads((GOLDEN / "trajectories.json").read_text())


@pytest.fixture(scope="session")
def oracle_runs():
    return json.loads((GOLDEN / "oracle_runs.json").read_text())


def load_npz(name):
    return np.load(GOLDEN / name, allow_pickle=False)

import os
import sys

os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger CPU cases")


@pytest.fixture(scope="session")
def golden_plm():
    return np.load(GOLDEN / "plm_golden.npz")


@pytest.fixture(scope="session")
def golden_skip():
    return np.load(GOLDEN / "ring_skip.npz")


def rel_alm_err(a, ref):
    """max_{l,m} |a - ref| / max |ref|, per map, then the max over maps
    (the alm error metric used for the parity bars)."""
    a = np.asarray(a)
    ref = np.asarray(ref)
    nsim = ref.shape[0]
    d = np.abs(a - ref).reshape(nsim, -1).max(axis=1)
    s = np.abs(ref).reshape(nsim, -1).max(axis=1)
    return float((d / np.maximum(s, 1e-300)).max())


def rel_map_err(a, ref):
    """max |a - ref| / std(ref) (the reference's map metric, scripts/demo.py:119)."""
    a = np.asarray(a)
    ref = np.asarray(ref)
    return float(np.abs(a - ref).max() / max(ref.std(), 1e-300))

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture
def golden():
    return load_golden


def rel_err(a, b, axis=None):
    """Normwise relative error ||a - b|| / ||b|| (per row when axis is given)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if axis is None:
        return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)
    num = np.sqrt(np.sum(np.abs(a - b) ** 2, axis=axis))
    den = np.sqrt(np.sum(np.abs(b) ** 2, axis=axis))
    return num / np.maximum(den, 1e-300)

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        'markers', 'gpu: needs a CUDA GPU and the built qsx library')


@pytest.fixture(scope='session')
def golden():
    path = os.path.join(ROOT, 'tests', 'golden', 'reference_golden.npz')
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope='session')
def golden_zofe_hermit():
    path = os.path.join(ROOT, 'tests', 'golden', 'reference_golden_zofe_hermit.npz')
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def rel_err(a, b):
    """max|a - b| / max|b| (the inf-norm relative error used by every test)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def as_matrix(d):
    return np.array(d["re"], dtype=np.float64) + 1j * np.array(d["im"], dtype=np.float64)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(params=["float_pairs", "fp64"])
def minors_arith(request):
    """Runs a test under both arithmetics of the all-minors sweeps, restoring the
    previous one afterwards."""
    from theboss_gb300 import _native

    mode = _native.FLOAT_PAIRS if request.param == "float_pairs" else _native.FP64
    prev = _native.minors_arithmetic(mode)
    yield request.param
    _native.minors_arithmetic(prev)

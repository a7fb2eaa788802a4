import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def bklib():
    """The CUDA library (built on demand, never skipped: the product has no
    CPU fallback)."""
    import omp_bk_gb300 as bk
    if not os.path.exists(bk.LIB_PATH):
        from omp_bk_gb300 import build
        build.build()
    bk.lib()
    return bk


@pytest.fixture(scope="session")
def golden():
    import json

    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")
    arrays = dict(np.load(os.path.join(d, "golden.npz")))
    meta = json.load(open(os.path.join(d, "golden.json")))
    return arrays, meta

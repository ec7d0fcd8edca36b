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
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def case_from_npz(z):
    from ibemproject_gb300.cases import Case
    return Case(float(z["E0"]), float(z["nu0"]), float(z["E1"]), float(z["nu1"]), z["nodes"],
                z["conn"].astype(np.int32), z["bc"], z["tbc"], z["centers"], z["radius"], z["points"])


def scaled_err(a, b):
    """max |a - b| / max |b| (entry error scaled by the largest reference entry)."""
    a = np.asarray(a)
    b = np.asarray(b)
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0))

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def seed_of(*key) -> int:
    """A seed fixed by the test parameters (Python's own hash() of strings changes per process)."""
    import zlib
    return zlib.crc32(repr(key).encode())


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    den = np.linalg.norm(b)
    if den == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / den)


def load_cases(name):
    """Group a golden .npz into {case_key: {field: array}}."""
    z = np.load(os.path.join(GOLDEN, name))
    cases = {}
    for k in z.files:
        case, field = k.split("__", 1)
        cases.setdefault(case, {})[field] = z[k]
    return cases


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle

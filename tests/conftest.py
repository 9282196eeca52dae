import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def reference_path(*parts):
    """A path inside the reference checkout named by DUGKS_REFERENCE_ROOT, or
    "" when the variable is unset (tests that read the reference's own demo
    cases in place skip then)."""
    root = os.environ.get("DUGKS_REFERENCE_ROOT", "")
    return os.path.join(root, *parts) if root else ""


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libdugks on cuda:0)")


@pytest.fixture(scope="session")
def built_lib():
    from dugksfoam_gb300 import build

    return build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle

    return oracle.build()


def rel_err(a, b):
    """max |a-b| / max |b| (field-normalised L-inf) and L2 analogue."""
    import numpy as np

    a = np.asarray(a, float)
    b = np.asarray(b, float)
    d = np.abs(a - b)
    r = np.abs(b)
    if a.ndim == 2:  # vector fields: magnitudes of the difference and of the reference
        d = np.linalg.norm(a - b, axis=1)
        r = np.linalg.norm(b, axis=1)
    return d.max() / r.max(), np.linalg.norm(d) / np.linalg.norm(r)

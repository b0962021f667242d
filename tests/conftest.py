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
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def golden_json():
    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        return json.load(fh)


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle():
    from oracle import lf_oracle
    lf_oracle.build()
    return lf_oracle


@pytest.fixture(scope="session")
def native():
    """The built liblfgpu binding (built on demand; never a fallback)."""
    from lightfem_gb300 import build
    build.build()
    from lightfem_gb300 import _native
    _native.library()
    return _native

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    here = os.path.join(ROOT, "tests", "golden")
    return {
        "ref": dict(np.load(os.path.join(here, "ks1d_reference_data.npz"))),
        "oracle": dict(np.load(os.path.join(here, "ks1d_oracle.npz"))),
        "ksr": dict(np.load(os.path.join(here, "ksr_h2.npz"))),
    }

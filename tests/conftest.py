import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "sph-multiphase_gb300"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library on cuda:0)")
    config.addinivalue_line("markers", "slow: full-size workload")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library and the oracle once per session."""
    from sphmp import build as B
    B.build()
    from oracle import oracle as O
    O.build()
    return True

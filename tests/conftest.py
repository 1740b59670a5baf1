"""Shared test setup: the `gpu` marker, import paths for the oracle and the
library binding, and session-scoped builds."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "math-atlas_gb300"))
GOLDEN = os.path.join(ROOT, "tests", "golden", "atlas_ref_fixtures.npz")
GOLDEN_LARGE = os.path.join(ROOT, "tests", "golden", "atlas_ref_large.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def ora():
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def golden_large():
    """Reference results at the headline sizes (pivots of the reference's own
    ATL_getrfC at n = 2048, 4096, 8192, FP32 pivots at 4096, sampled entries
    of the reference BLAS DGEMM at 1024^3)."""
    import numpy as np
    return np.load(GOLDEN_LARGE)


@pytest.fixture(scope="session")
def gb():
    import atlas_gb300
    if not os.path.exists(atlas_gb300.LIB_PATH):
        atlas_gb300.build()
    atlas_gb300.lib()
    return atlas_gb300

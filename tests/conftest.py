import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def solver_lib():
    """The CUDA solver library, built in-tree if needed (incremental)."""
    from fluidx3d_gb300 import build, _capi
    build.build()
    return _capi.load()


@pytest.fixture(scope="session")
def gpu(solver_lib):
    """Skips when no CUDA device is present; any other failure is an error."""
    from fluidx3d_gb300 import LBM, LBMError
    try:
        lbm = LBM(4, 4, 4, 0.1)
        lbm.close()
    except LBMError as e:
        if e.status == 6:
            pytest.skip("no CUDA device")
        raise
    return True


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")

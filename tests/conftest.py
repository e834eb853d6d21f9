import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cyclosubfield-dbfv_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs through the C-ABI library")
    config.addinivalue_line("markers", "slow: full-size CPU oracle runs (seconds to minutes)")


@pytest.fixture(scope="session")
def po():
    from oracle import pyoracle

    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def be():
    import halcuda

    backend = halcuda.CudaBackend(0)
    yield backend
    backend.close()

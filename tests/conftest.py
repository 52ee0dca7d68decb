import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    from oracle import Port

    Port.lib()
    return Port


@pytest.fixture(scope="session")
def gpu_lib():
    import mlau_gb300 as M
    from mlau_gb300 import _build

    _build.build()  # no-op when the in-tree library is up to date
    M.lib()
    return M


@pytest.fixture(scope="session", autouse=True)
def _fresh_library():
    from mlau_gb300 import _build

    _build.build()

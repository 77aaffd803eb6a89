import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libHYPRE_gb300.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gb():
    import hypre_gb300
    hypre_gb300.lib().HYPRE_Initialize()
    return hypre_gb300


@pytest.fixture(autouse=True)
def _clear_error_flag(request):
    """Each test starts with a clear sticky error flag (as a fresh process would)."""
    if "gb" in request.fixturenames:
        import hypre_gb300
        hypre_gb300.lib().HYPRE_ClearAllErrors()
    yield

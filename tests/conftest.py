import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
PKG = os.path.join(ROOT, "rust-la_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def lagpu():
    """The CUDA library, built in-tree if needed. Fails loudly when it cannot load."""
    import build as pkg_build
    pkg_build.build()
    import la_gpu
    la_gpu.lib()
    return la_gpu


@pytest.fixture(scope="session")
def ctx_fast(lagpu):
    c = lagpu.Context(arith=lagpu.ARITH_FAST)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ctx_exact(lagpu):
    c = lagpu.Context(arith=lagpu.ARITH_EXACT)
    yield c
    c.close()

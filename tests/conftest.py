import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "blaze-sc-ad_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libblaze103")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session", autouse=True)
def built_library():
    """Builds libblaze103 (nvcc, sm_103a) when a fresh checkout runs the tests
    before the build step; the library itself never falls back to anything."""
    if not os.path.exists(os.path.join(PKG, "blaze103", "libblaze103.so")):
        import build as pkg_build  # blaze-sc-ad_gb300/build.py

        pkg_build.build()

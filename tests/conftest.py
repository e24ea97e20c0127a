import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "axion-strings_gb300")
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (PKG, TESTS, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI of libaxs.so")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib.load()


@pytest.fixture(scope="session")
def axs():
    """The product module. On a GPU run a missing build is an error, not a skip."""
    lib = os.path.join(PKG, "libaxs.so")
    if not os.path.exists(lib):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py")], check=True)
    import axs as mod
    return mod

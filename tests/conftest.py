import glob
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "p4-phylogenetics_gb300")
for p in (PKG, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libp4gpu.so")


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def golden_ids():
    return [os.path.basename(f)[:-4] for f in golden_files()]


@pytest.fixture(scope="session")
def lib():
    """libp4gpu.so, built in-tree if missing."""
    from p4gpu import _lib
    if not os.path.exists(_lib.LIB_PATH):
        sys.path.insert(0, PKG)
        import build as _b
        _b.build()
    return _lib.load()


@pytest.fixture(scope="session")
def port():
    from oracle import oracle
    oracle.port_lib()
    return oracle

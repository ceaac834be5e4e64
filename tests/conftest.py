import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.bind import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def lib():
    """The product library, built in-tree if needed."""
    import libfmftsaxs_gb300 as g
    from libfmftsaxs_gb300 import build
    if not os.path.exists(g.LIB_PATH):
        build.build()
    g.load()
    return g


@pytest.fixture(scope="session")
def gpu(lib):
    lib.init(0)
    return lib


@pytest.fixture(scope="session")
def ref():
    from oracle.bind import Ref, have_ref
    if not have_ref():
        pytest.skip("no reference build: set FMFTSAXS_REFERENCE_SRC to the reference source tree")
    return Ref()

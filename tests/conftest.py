import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# A device failure inside a Fortran-ABI call prints and returns instead of
# aborting the whole test process, so the failing test is reported.
os.environ.setdefault("BLAS2CUDA_OPTIONS", "errors=return")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.get()


@pytest.fixture(scope="session")
def cpublas():
    from oracle import cpublas as cb
    return cb.get()


@pytest.fixture(scope="session")
def lib():
    """The built library; building it is part of the session setup."""
    from libgpublas_gb300 import build
    build.build_library()
    import libgpublas_gb300 as g
    return g.load()


@pytest.fixture(scope="session")
def f77(lib):
    import libgpublas_gb300 as g
    return g.F77()


@pytest.fixture(scope="session")
def dev(lib):
    import libgpublas_gb300 as g
    d = g.Device(0)
    yield d
    d.close()

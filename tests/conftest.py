import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product library's kernels")


@pytest.fixture(scope="session")
def built():
    """Builds the product library and the oracle once per session."""
    import __graft_entry__ as g
    from hpc_gb300 import build as B
    import oracle
    B.build_library()
    oracle.build()
    return g


@pytest.fixture(scope="session")
def gpu_lib(built):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    import hpc_gb300 as X
    return X.load()


@pytest.fixture()
def handle(gpu_lib):
    import hpc_gb300 as X
    h = X.JPCG()
    yield h
    h.close()

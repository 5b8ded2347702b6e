import importlib
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("2d_dvm_microflows_gb300")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpulib(pkg):
    """The C-ABI library, built in-tree if missing; skips without a GPU."""
    if not os.path.exists(pkg.LIB_PATH):
        b = importlib.import_module("2d_dvm_microflows_gb300.build")
        b.build()
    lib = pkg.load_library()
    import torch
    if torch.cuda.device_count() < 1:
        pytest.fail("no CUDA device visible to a gpu-marked test")
    return lib

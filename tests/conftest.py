import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300)")


def pytest_collection_modifyitems(config, items):
    import torch

    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built_lib():
    """The CUDA library, built in-tree if missing (compilation needs only nvcc)."""
    from supernormal_gb300 import _lib, build

    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.lib()


@pytest.fixture(scope="session")
def dev():
    import torch

    return torch.device("cuda:0")

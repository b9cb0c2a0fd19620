import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    import orc as _orc
    _orc.lib()
    return _orc


@pytest.fixture(scope="session")
def sadlib():
    """libsad_gb300.so, built from source if it is missing or stale."""
    from sad_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda(sadlib):
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("GPU tests need a CUDA device")
    return torch.device("cuda", 0)

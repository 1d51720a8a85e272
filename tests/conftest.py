import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mflops3d-md_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _lib_built():
    return os.path.exists(os.path.join(PKG, "lib", "libmflops_gb300.so"))


@pytest.fixture(scope="session")
def mf():
    if not _lib_built():
        import build  # noqa: F401  (mflops3d-md_gb300/build.py)
        build.build()
    import mflops_gb300
    return mflops_gb300


@pytest.fixture(scope="session")
def gpu(mf):
    import torch
    if not torch.cuda.is_available() or not mf.device_available():
        pytest.fail("GPU test collected without a usable CUDA device")
    return torch

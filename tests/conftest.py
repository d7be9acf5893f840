import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "concrete-fft_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session")
def cfft_lib():
    """The product library, built in-tree if it is missing (nvcc cross-compiles on CPU hosts)."""
    import build as pkg_build  # concrete-fft_gb300/build.py
    if not os.path.exists(pkg_build.LIB):
        pkg_build.build()
    import concrete_fft
    return concrete_fft.load()


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def cuda(cfft_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import concrete_fft
    concrete_fft.check(cfft_lib.cfft_device_check())
    return torch


def bits(x):
    """Bit pattern of a float64/complex128 array, for exact comparisons."""
    import numpy as np
    x = np.ascontiguousarray(x)
    return x.view(np.uint64)

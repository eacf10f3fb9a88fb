import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "acoustic-field-calculator_gb300")
for p in (PKG, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def lib_path():
    import build_lib

    return build_lib.build()


@pytest.fixture(scope="session")
def afc_mod(lib_path):
    import afc

    return afc


@pytest.fixture(scope="session")
def has_gpu(afc_mod):
    return afc_mod.DLL.AFC_CudaDeviceCount() > 0


@pytest.fixture(scope="session")
def gpu(afc_mod, has_gpu):
    if not has_gpu:
        pytest.fail("a test marked gpu ran without a usable CUDA device")
    return afc_mod

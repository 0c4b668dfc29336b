import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built voxelis_gb300 library")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as oracle_build
    from voxelis_gb300._abi import NativeLib

    return NativeLib(oracle_build.build(), "vxo_")


@pytest.fixture(scope="session")
def gpu_lib():
    from voxelis_gb300._abi import gpu_lib as load

    return load()


@pytest.fixture(params=["oracle", pytest.param("gpu", marks=pytest.mark.gpu)])
def lib(request):
    """The library under test: the CPU oracle (always) and the GPU library (gpu-marked runs)."""
    return request.getfixturevalue(request.param + "_lib")

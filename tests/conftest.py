"""Shared fixtures.  Tests that need a GPU are marked ``gpu``; everything
else runs on the CPU (oracle, host logic, library load and argument checks)."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def built_library():
    """Path of the CUDA library, compiled here if missing (nvcc cross-compiles)."""
    from stonefish_gb300 import abi, build
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    return abi.LIB_PATH


@pytest.fixture(scope="session")
def hctx(built_library):
    """Default context: FP32 cut points in the reference's operation order."""
    from stonefish_gb300 import abi
    from stonefish_gb300.hydro import HydroContext
    h = HydroContext()
    assert h.cut_precision == abi.CUT_FP32
    yield h
    h.close()


@pytest.fixture(scope="session")
def hctx64(built_library):
    """Context with FP64 cut points."""
    from stonefish_gb300 import abi
    from stonefish_gb300.hydro import HydroContext
    h = HydroContext(cut_precision=abi.CUT_FP64)
    yield h
    h.close()

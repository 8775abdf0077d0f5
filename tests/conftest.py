import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs through the C ABI of libcvl_gb300.so)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import HostRunner, load_oracle
    return HostRunner(load_oracle())


@pytest.fixture(scope="session")
def reference():
    from oracle.oracle import HostRunner, load_reference
    ref = load_reference()
    if ref is None:
        pytest.skip("reference serial CVL not built here (needs the reference tree)")
    return HostRunner(ref)


def _has_gpu() -> bool:
    try:
        import ctypes
        cudart = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int(0)
        if cudart.cuInit(0) != 0:
            return False
        return cudart.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not _has_gpu():
        pytest.skip("no GPU")
    from neslgpu_gb300.ops import DeviceRunner
    from neslgpu_gb300.cvl import load
    return DeviceRunner(load())

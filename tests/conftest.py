import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcuda.so.1", "libcuda.so"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        n = ctypes.c_int(0)
        if cudart.cuInit(0) != 0:
            return False
        return cudart.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def native():
    """The built libgbpt.so (built on demand; the GPU tests need it on the GPU machine)."""
    from merian_gb300 import build, _native
    build.build()
    return _native.load()


@pytest.fixture(scope="session")
def gpu_ctx(native):
    if not HAS_GPU:
        pytest.fail("GPU test collected on a machine without a CUDA device")
    from merian_gb300.scene import Context
    ctx = Context(0)
    yield ctx
    ctx.close()

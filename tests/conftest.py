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


def facing_case(axis: int, sign: float):
    """A one-sided triangle in the plane (axis) = 0, counter-clockwise seen from the + side, four
    times: as given (instance mask 1), wound the other way (2), with FlipFacing (4) and TwoSided
    (8); one off-axis ray along -sign * axis from the sign side. Returns (scene, rays, {mask:
    expected hit}, expected t)."""
    import numpy as np
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    u, w = (axis + 1) % 3, (axis + 2) % 3
    tri = np.zeros((3, 3))
    tri[1, u] = 1.0
    tri[2, w] = 1.0
    v = np.zeros(6, N.VERTEX_DTYPE)
    v["position"][:3] = tri
    v["position"][3:] = tri[[0, 2, 1]]
    g = np.zeros(4, N.GEOMETRY_DTYPE)
    g["first_vertex"] = [0, 3, 0, 3]
    g["triangle_count"] = 1
    g["flags"] = [0, 0, N.MESH_FLIP_FACING, N.MESH_TWO_SIDED]
    g["instance_mask"] = [1, 2, 4, 8]
    m = np.zeros(1, N.MATERIAL_DTYPE)
    m["model"] = N.MATERIAL_DIFFUSE
    m["base_color"] = 0.5
    m["specular_alpha"] = 1.0
    m["specular_ior"] = 1.5
    m["base_color_texture"] = -1
    m["alpha_texture"] = -1
    sc = S.SceneData(v, np.array([[0, 1, 2]], np.uint32), g, m, None)
    rays = np.zeros(1, N.RAY_DTYPE)
    o = np.full(3, 0.25)
    o[axis] = 2.0 * sign
    d = np.zeros(3)
    d[axis] = -sign
    d[u], d[w] = 0.01, -0.02  # off-axis, so the 2D frame is a real shear
    rays["origin"], rays["direction"], rays["tmax"] = o, d, 1e30
    front = sign > 0
    return sc, rays, {1: front, 2: not front, 4: not front, 8: True}, 2.0

"""CPU tests of the C ABI: the library loads, exports every declared entry point, and its host-only
helpers (scene generators, encodings, camera basis) behave. No device work."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import HAS_GPU, ROOT

HEADER = ROOT / "include" / "gbpt.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"GBPT_API\s+[\w\s\*]+?\b(gbpt_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gbpt_render" in syms and "gbpt_scene_create" in syms and len(syms) >= 18


def test_library_exports_every_declared_symbol(native):
    from merian_gb300 import _native as N
    bound = {name for name, _, _ in N.EXPORTS}
    for s in declared_symbols():
        assert hasattr(native, s), f"{s} not exported by libgbpt.so"
        assert s in bound, f"{s} has no ctypes prototype"


def test_abi_version(native):
    # 2: gbpt_tuning's traversal schedule fields, gbpt_render_stats' SIMT step counts
    assert native.gbpt_abi_version() == 2
    from merian_gb300 import _native as N
    assert C.sizeof(N.Tuning) == 40 and C.sizeof(N.RenderStats) == 136


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device error path")
def test_create_fails_loudly_without_a_device(native):
    h = C.c_void_p()
    rc = native.gbpt_create(0, 0, C.byref(h))
    assert rc != 0 and not h.value
    assert native.gbpt_last_error()


def test_cornell_generator_sizes_and_determinism(native):
    from merian_gb300 import scene as S
    a, b = S.cornell(), S.cornell()
    assert len(a.vertices) == 3072 and a.indices.shape == (1024, 3)
    assert a.geometries["triangle_count"].sum() == 1024
    assert sorted(a.geometries["material_id"]) == list(range(8))
    for k in ("vertices", "indices", "geometries", "materials"):
        assert getattr(a, k).tobytes() == getattr(b, k).tobytes()
    em = a.materials[a.materials["emission"][:, 0] > 0]
    assert len(em) == 1 and np.all(em["emission"] == 15.0)
    light = a.geometries[a.geometries["material_id"] == 7][0]
    assert light["triangle_count"] == 8
    # the emitter is the centre 0.25 x 0.25 of the ceiling, facing down
    tri = a.indices[light["first_triangle"]:light["first_triangle"] + 8]
    p = a.vertices["position"][tri.reshape(-1)]
    assert np.allclose(p[:, 1], 1.0)
    assert np.isclose(p[:, 0].min(), 0.375) and np.isclose(p[:, 0].max(), 0.625)
    e1 = p[1] - p[0]
    e2 = p[2] - p[0]
    assert np.cross(e1, e2)[1] < 0
    albedo = a.materials["base_color"][:7]
    assert np.all((albedo >= 0.2) & (albedo <= 0.8))


def test_cornell_matches_golden_scene(native):
    from merian_gb300 import scene as S
    sys_path = ROOT / "tests" / "golden"
    import sys
    sys.path.insert(0, str(sys_path))
    from make_golden import scene_hash
    g = np.load(ROOT / "tests" / "golden" / "cornell.npz")
    assert scene_hash(S.cornell()) == str(g["scene_hash"])


def test_soup_generator(native):
    from merian_gb300 import scene as S
    a = S.soup(7, 3000, 30, (64, 32))
    b = S.soup(7, 3000, 30, (64, 32))
    assert a.vertices.tobytes() == b.vertices.tobytes() and a.env.tobytes() == b.env.tobytes()
    p = a.vertices["position"].reshape(-1, 3, 3)
    c = p.mean(axis=1)
    assert np.all(c > -0.2) and np.all(c < 1.2)
    edge = np.linalg.norm(p[:, 1] - p[:, 0], axis=1)
    assert 0.005 < np.median(edge) < 0.03
    models = a.materials["model"]
    assert set(np.unique(models)) <= {0, 1, 2}
    assert np.all(a.geometries["flags"] & 0x10)
    assert a.env.shape == (32, 64, 4) and np.all(a.env[..., :3] > 0)


def test_encode_normal_roundtrip_and_half(native):
    rng = np.random.default_rng(1)
    n = rng.normal(size=(200, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    for v in n:
        enc = native.gbpt_encode_normal((C.c_float * 3)(*v))
        x = float(np.array(enc & 0xFFFF, np.uint16).view(np.int16)) / 32767.0
        y = float(np.array(enc >> 16, np.uint16).view(np.int16)) / 32767.0
        z = 1 - abs(x) - abs(y)
        if z < 0:
            x, y = np.copysign(1 - abs(y), x), np.copysign(1 - abs(x), y)
        d = np.array([x, y, z])
        d /= np.linalg.norm(d)
        assert np.dot(d, v) > 1 - 1e-6
    for a, b in [(0.1, 0.7), (1e-6, 65504.0), (0.33333, -2.5)]:
        h = native.gbpt_pack_half2(a, b)
        assert np.float16(a).view(np.uint16) == (h & 0xFFFF)
        assert np.float16(b).view(np.uint16) == (h >> 16)


def test_camera_basis_matches_merian_formula(native):
    from merian_gb300 import scene as S
    cam = S.look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.0), (0, 1, 0), 40.0, 2.0, 0.1, 1000.0)
    pos, tgt, up = np.array([0.5, 0.5, -1.4]), np.array([0.5, 0.5, 0.0]), np.array([0, 1, 0.0])
    fwd = (tgt - pos) / np.linalg.norm(tgt - pos)
    rgt = np.cross(fwd, up)
    rgt /= np.linalg.norm(rgt)
    focus = np.linalg.norm(tgt - pos)
    ht = np.tan(np.radians(40.0) / 2)
    assert np.allclose(list(cam.U), rgt * ht * 2.0 * focus, atol=1e-6)
    assert np.allclose(list(cam.V), np.cross(rgt, fwd) * ht * focus, atol=1e-6)
    assert np.allclose(list(cam.W), fwd * focus, atol=1e-6)
    assert cam.near_plane == pytest.approx(0.1) and cam.far_plane == pytest.approx(1000.0)

"""glTF 2.0 loading (gbpt_load_gltf), following merian's GLTFScene
(src/merian-shaders/scene/gltf_scene.cpp).

Files are written here: a .gltf with an external .bin and a PNG image file, the same scene as a
.glb with the buffer and the image embedded, and a .gltf with data-URI buffers. Checked against
what the files say: mesh -> BLAS, node -> instance with its world transform (matrix and TRS,
parent chains), the perspective camera, materials mapped onto the OpenPBR record, alphaMode MASK
-> alpha test on the base colour texture, doubleSided / transmission -> two-sided, PNG texels.
GPU: primary hits of the loaded scene bit-identical to the FP32 oracle.
"""
import base64
import json
import math
import struct

import numpy as np
import pytest

from oracle import binding as O
from test_png import write_png


def _quat(axis, deg):
    a = np.asarray(axis, float) / np.linalg.norm(axis)
    h = math.radians(deg) / 2
    return [*(a * math.sin(h)), math.cos(h)]


def build_scene(tmp_path, kind):
    """kind: 'gltf' (external .bin + .png), 'glb' (embedded), 'datauri'."""
    # mesh 0: a quad (indexed, normals, uvs); mesh 1: a tetrahedron (no indices, no normals)
    quad_p = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
    quad_n = np.tile(np.array([0, 0, 1], np.float32), (4, 1))
    quad_uv = np.array([[0, 1], [1, 1], [1, 0], [0, 0]], np.float32)
    quad_i = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    tet = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 0], [0, 1, 0], [0, 0, 1],
                    [0, 0, 0], [0, 0, 1], [1, 0, 0], [1, 0, 0], [0, 0, 1], [0, 1, 0]], np.float32)
    blobs = [quad_p.tobytes(), quad_n.tobytes(), quad_uv.tobytes(), quad_i.tobytes() + b"\0\0",
             tet.tobytes()]
    offs = np.cumsum([0] + [len(b) for b in blobs])
    binary = b"".join(blobs)
    # an 8 x 8 texture: opaque checkerboard cells with alpha 255 / 0
    i, j = np.meshgrid(np.arange(8), np.arange(8), indexing="ij")
    tex = np.zeros((8, 8, 4), np.uint8)
    tex[..., 0] = 40 + 20 * i
    tex[..., 1] = 200 - 10 * j
    tex[..., 2] = 90
    tex[..., 3] = np.where((i + j) % 2 == 0, 255, 0)
    write_png(tmp_path / "tex.png", tex.reshape(8, 32), 6, 8, 9)
    png = (tmp_path / "tex.png").read_bytes()

    views = [{"buffer": 0, "byteOffset": int(offs[k]), "byteLength": len(blobs[k])}
             for k in range(5)]
    views[3]["byteLength"] = 12
    acc = [
        {"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
        {"bufferView": 1, "componentType": 5126, "count": 4, "type": "VEC3"},
        {"bufferView": 2, "componentType": 5126, "count": 4, "type": "VEC2"},
        {"bufferView": 3, "componentType": 5123, "count": 6, "type": "SCALAR"},
        {"bufferView": 4, "componentType": 5126, "count": 12, "type": "VEC3"},
    ]
    image = {"uri": "tex.png"}
    doc = {
        "asset": {"version": "2.0"},
        "scene": 0,
        "scenes": [{"nodes": [0, 3, 4]}],
        "nodes": [
            {"translation": [0, 0, -2], "children": [1, 2]},
            {"mesh": 0, "rotation": _quat([0, 1, 0], 30), "scale": [2, 2, 2]},
            {"mesh": 1, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 3, 0, 0, 1]},
            {"mesh": 1, "translation": [-3, 0, -1]},
            {"camera": 0, "translation": [0, 0, 6]},
        ],
        "meshes": [
            {"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2},
                             "indices": 3, "material": 0}]},
            {"primitives": [{"attributes": {"POSITION": 4}, "material": 1}]},
        ],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorFactor": [0.8, 0.6, 0.4, 1.0],
                                      "baseColorTexture": {"index": 0},
                                      "metallicFactor": 0.0, "roughnessFactor": 0.5},
             "alphaMode": "MASK", "doubleSided": True},
            {"pbrMetallicRoughness": {"baseColorFactor": [1, 1, 1, 1], "metallicFactor": 0.0,
                                      "roughnessFactor": 0.1},
             "emissiveFactor": [1, 0.5, 0.25],
             "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 4},
                            "KHR_materials_transmission": {"transmissionFactor": 1},
                            "KHR_materials_ior": {"ior": 1.33}}},
        ],
        "textures": [{"source": 0}],
        "images": [image],
        "cameras": [{"type": "perspective",
                     "perspective": {"yfov": 0.7, "aspectRatio": 1.5, "znear": 0.1}}],
        "accessors": acc,
        "bufferViews": views,
        "buffers": [{"byteLength": len(binary), "uri": "scene.bin"}],
    }
    if kind == "gltf":
        (tmp_path / "scene.bin").write_bytes(binary)
        path = tmp_path / "scene.gltf"
        path.write_text(json.dumps(doc))
    elif kind == "datauri":
        doc["buffers"][0]["uri"] = ("data:application/octet-stream;base64," +
                                    base64.b64encode(binary).decode())
        doc["images"][0] = {"uri": "data:image/png;base64," + base64.b64encode(png).decode()}
        path = tmp_path / "scene_datauri.gltf"
        path.write_text(json.dumps(doc))
    else:
        pad = (-len(binary)) % 4
        img_off = len(binary) + pad
        binary = binary + b"\0" * pad + png
        doc["bufferViews"].append({"buffer": 0, "byteOffset": img_off, "byteLength": len(png)})
        doc["images"][0] = {"bufferView": 5, "mimeType": "image/png"}
        del doc["buffers"][0]["uri"]
        doc["buffers"][0]["byteLength"] = len(binary)
        js = json.dumps(doc).encode()
        js += b" " * ((-len(js)) % 4)
        binary += b"\0" * ((-len(binary)) % 4)
        body = (struct.pack("<II", len(js), 0x4E4F534A) + js +
                struct.pack("<II", len(binary), 0x004E4942) + binary)
        path = tmp_path / "scene.glb"
        path.write_bytes(struct.pack("<4sII", b"glTF", 2, 12 + len(body)) + body)
    return path, tex


def _rot_y(deg):
    c, s = math.cos(math.radians(deg)), math.sin(math.radians(deg))
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


@pytest.mark.parametrize("kind", ["gltf", "glb", "datauri"])
def test_gltf_structure(native, tmp_path, kind):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    path, tex = build_scene(tmp_path, kind)
    sc, cam, (w, h), warnings = S.load_gltf(path)
    assert (w, h) == (1080, 720)
    assert list(sc.geometries["triangle_count"]) == [2, 4]
    assert list(sc.blas_ranges["first_geometry"]) == [0, 1]
    # instances in node order: node 1 (quad), node 2 (tet), node 3 (tet)
    assert list(sc.instances["blas"]) == [0, 1, 1]
    m = sc.instances["object_to_world"].reshape(-1, 3, 4)
    assert np.allclose(m[0][:, :3], 2 * _rot_y(30), atol=1e-6)
    assert np.allclose(m[0][:, 3], [0, 0, -2])
    assert np.allclose(m[1], [[1, 0, 0, 3], [0, 1, 0, 0], [0, 0, 1, -2]])
    assert np.allclose(m[2], [[1, 0, 0, -3], [0, 1, 0, 0], [0, 0, 1, -1]])
    g = sc.geometries
    assert g["flags"][0] & N.MESH_ALPHA_TEST and g["flags"][0] & N.MESH_TWO_SIDED
    assert g["flags"][1] & N.MESH_TWO_SIDED and not g["flags"][1] & N.MESH_ALPHA_TEST
    m0, m1 = sc.materials[g["material_id"]]
    assert np.allclose(m0["base_color"], [0.8, 0.6, 0.4]) and m0["metalness"] == 0
    assert np.isclose(m0["specular_alpha"][0], 0.25)
    assert m0["base_color_texture"] == 0 and m0["alpha_texture"] == 0
    assert m1["model"] == N.MATERIAL_OPENPBR_TRANSMISSION and np.isclose(m1["specular_ior"], 1.33)
    assert np.allclose(m1["emission"], [4, 2, 1]) and np.isclose(m1["specular_alpha"][0], 0.01)
    assert len(sc.textures) == 1 and sc.textures[0][1] is True
    assert np.array_equal(sc.textures[0][0], tex)
    # smooth normals of the unindexed tetrahedron, given normals of the quad
    n = sc.vertices["encoded_normal"]
    assert np.all(n[:4] == n[0])
    # camera: at (0, 0, 6) looking down -z, yfov 0.7
    ref = N.Camera()
    f3 = N.C.c_float * 3
    N.check(N.load().gbpt_camera_look_at(f3(0, 0, 6), f3(0, 0, 5), f3(0, 1, 0), 0.7, 1.5, 0.1,
                                         1000.0, N.C.byref(ref)))
    for f in ("position", "U", "V", "W"):
        assert np.allclose(np.array(getattr(cam, f)), np.array(getattr(ref, f)), atol=1e-6), f


def test_gltf_through_oracle(native, tmp_path):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    path, _ = build_scene(tmp_path, "glb")
    sc, cam, (w, h), _ = S.load_gltf(path)
    hits, _ = O.OracleScene(sc).trace_primary(cam, 216, 144, fp64=False, hit_dtype=N.HIT_DTYPE)
    hit = hits["t"] > 0
    seen = set(hits["instance_index"][hit].tolist())
    assert seen == {0, 1, 2}
    # the masked quad shows holes: fewer quad hits than with the mask off
    opaque = S.load_gltf(path)[0]
    opaque.geometries["flags"] &= ~np.uint32(N.MESH_ALPHA_TEST)
    h2, _ = O.OracleScene(opaque).trace_primary(cam, 216, 144, fp64=False, hit_dtype=N.HIT_DTYPE)
    q1 = np.sum(hits["instance_index"][hit] == 0)
    q2 = np.sum(h2["instance_index"][h2["t"] > 0] == 0)
    assert 0.3 * q2 < q1 < 0.7 * q2


def test_gltf_errors(native, tmp_path):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    (tmp_path / "a.gltf").write_text('{"asset": {"version": "2.0"}, "meshes": [')
    with pytest.raises(N.GbptError, match="JSON"):
        S.load_gltf(tmp_path / "a.gltf")
    (tmp_path / "b.gltf").write_text('{"asset": {"version": "2.0"}}')
    with pytest.raises(N.GbptError, match="no meshes"):
        S.load_gltf(tmp_path / "b.gltf")
    path, _ = build_scene(tmp_path, "gltf")
    (tmp_path / "scene.bin").write_bytes(b"\0" * 10)
    with pytest.raises(N.GbptError):
        S.load_gltf(path)
    with pytest.raises(N.GbptError):
        S.load_gltf(tmp_path / "missing.glb")


@pytest.mark.gpu
def test_gltf_scene_on_gpu(gpu_ctx, tmp_path):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    path, _ = build_scene(tmp_path, "glb")
    sc, cam, _, _ = S.load_gltf(path)
    sid = gpu_ctx.upload(sc)
    try:
        g = gpu_ctx.trace_primary(sid, cam, 216, 144)
        o, _ = O.OracleScene(sc).trace_primary(cam, 216, 144, fp64=False, hit_dtype=N.HIT_DTYPE)
        for k in ("instance_id", "instance_index", "geometry_index", "primitive_id"):
            assert np.array_equal(g[k], o[k]), k
        assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
    finally:
        gpu_ctx.destroy_scene(sid)

"""pbrt-v4 scene loading (gbpt_load_pbrt), following merian's PBRTScene
(src/merian-shaders/scene/pbrt_scene.cpp).

CPU: a scene file exercising every supported directive (transforms, attribute scopes, named and
inline materials of each supported type, area lights, constant infinite light, trianglemesh,
ASCII and binary PLY with quads, sphere, disk, object instancing, ReverseOrientation, Include) is
loaded and checked against what the file says; the loaded scene goes through the oracle.
GPU: the loaded scene's primary hits are bit-identical to the FP32 oracle and its render is
finite and lit.
"""
import math
import struct

import numpy as np
import pytest

from oracle import binding as O

SCENE = r"""
# a small pbrt-v4 scene
Film "rgb" "integer xresolution" [ 160 ] "integer yresolution" [ 90 ] "string filename" "x.exr"
LookAt 0 1 -5   0 0.5 0   0 1 0
Camera "perspective" "float fov" [ 40 ]
Sampler "zsobol" "integer pixelsamples" 16
Integrator "volpath" "integer maxdepth" [ 5 ]
ColorSpace "srgb"
Option "bool disablepixeljitter" true
WorldBegin
LightSource "infinite" "rgb L" [ 0.2 0.3 0.4 ] "float scale" 2
LightSource "point" "point3 from" [ 0 4 0 ]
Texture "checks" "spectrum" "checkerboard" "float uscale" 8
MakeNamedMaterial "gold" "string type" "conductor" "spectrum eta" "metal-Au-eta"
    "spectrum k" "metal-Au-k" "float roughness" 0.04
MakeNamedMaterial "rough" "string type" "coateddiffuse" "rgb reflectance" [ 0.7 0.1 0.1 ]
    "float roughness" 0.25 "float eta" 1.4
MakeNamedMaterial "glassy" "string type" "dielectric" "float eta" 1.33
MakeNamedMaterial "either" "string type" "mix" "string materials" [ "rough" "gold" ]
    "float amount" 0.7
AttributeBegin
  AreaLightSource "diffuse" "rgb L" [ 8 7 6 ] "float scale" 1.5
  Translate 0 3 0
  Shape "trianglemesh" "point3 P" [ -1 0 -1  1 0 -1  1 0 1  -1 0 1 ]
      "integer indices" [ 0 2 1  0 3 2 ]
AttributeEnd
AttributeBegin
  Material "diffuse" "rgb reflectance" [ 0.2 0.4 0.6 ]
  Shape "trianglemesh" "point3 P" [ -4 0 -4  4 0 -4  4 0 4  -4 0 4 ]
      "normal N" [ 0 1 0  0 1 0  0 1 0  0 1 0 ]
      "point2 uv" [ 0 0  1 0  1 1  0 1 ] "integer indices" [ 0 1 2  0 2 3 ]
AttributeEnd
AttributeBegin
  NamedMaterial "gold"
  Translate 1.5 0.5 0
  Shape "sphere" "float radius" 0.5
AttributeEnd
AttributeBegin
  NamedMaterial "glassy"
  Translate -1.5 0.5 0
  Scale -1 1 1
  Shape "plymesh" "string filename" "mesh_ascii.ply"
AttributeEnd
AttributeBegin
  NamedMaterial "either"
  ReverseOrientation
  Translate 0 0.01 1.5
  Rotate -90 1 0 0
  Shape "disk" "float radius" 0.4
AttributeEnd
Include "extra.pbrt"
Texture "leaves" "spectrum" "imagemap" "string filename" "leaf.png" "float scale" 0.8
AttributeBegin
  Material "diffuse" "texture reflectance" "leaves"
  Translate 0 2 2
  Shape "trianglemesh" "point3 P" [ -1 0 0  1 0 0  1 1 0  -1 1 0 ]
      "point2 uv" [ 0 0  1 0  1 1  0 1 ] "integer indices" [ 0 1 2  0 2 3 ]
AttributeEnd
AttributeBegin
  Material "coateddiffuse" "texture reflectance" "checks"
  Shape "trianglemesh" "point3 P" [ 3 0 2  4 0 2  3 1 2 ]
AttributeEnd
ObjectBegin "tree"
  Material "conductor" "rgb reflectance" [ 0.9 0.8 0.7 ] "float uroughness" 0.09
      "float vroughness" 0.16 "bool remaproughness" false
  Shape "plymesh" "string filename" "mesh_binary.ply"
ObjectEnd
AttributeBegin
  Translate 0 0 3
  ObjectInstance "tree"
AttributeEnd
AttributeBegin
  Translate 2 0 3
  Rotate 90 0 1 0
  Scale 0.5 0.5 0.5
  ObjectInstance "tree"
AttributeEnd
"""

EXTRA = r"""
AttributeBegin
  Material "measured" "string filename" "x.bsdf"
  Shape "trianglemesh" "point3 P" [ -3 0 2  -2 0 2  -3 1 2 ]
AttributeEnd
Shape "curve" "point3 P" [ 0 0 0 1 1 1 2 2 2 3 3 3 ]
"""

# a unit square (one quad) and a triangle, ASCII
PLY_ASCII = """ply
format ascii 1.0
comment test mesh
element vertex 5
property float x
property float y
property float z
property float nx
property float ny
property float nz
property float u
property float v
element face 2
property list uchar int vertex_indices
end_header
0 0 0 0 0 -1 0 0
1 0 0 0 0 -1 1 0
1 1 0 0 0 -1 1 1
0 1 0 0 0 -1 0 1
0.5 1.5 0 0 0 -1 0.5 1
4 0 1 2 3
3 3 2 4
"""


def binary_ply(path):
    """A tetrahedron as binary_little_endian PLY (positions only: smooth normals computed)."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    f = [(0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3)]
    hdr = ("ply\nformat binary_little_endian 1.0\nelement vertex 4\nproperty float x\n"
           "property float y\nproperty float z\nelement face 4\n"
           "property list uchar int vertex_indices\nend_header\n").encode()
    body = v.tobytes() + b"".join(struct.pack("<B3i", 3, *t) for t in f)
    path.write_bytes(hdr + body)


@pytest.fixture(scope="module")
def pbrt_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("pbrt")
    (d / "scene.pbrt").write_text(SCENE)
    (d / "extra.pbrt").write_text(EXTRA)
    (d / "mesh_ascii.ply").write_text(PLY_ASCII)
    binary_ply(d / "mesh_binary.ply")
    from test_png import write_png
    leaf = np.zeros((4, 4, 4), np.uint8)
    leaf[..., 1] = 180
    leaf[..., 3] = np.where(np.arange(16).reshape(4, 4) % 3 == 0, 0, 255)
    write_png(d / "leaf.png", leaf.reshape(4, 16), 6, 8)
    return d


def _load(pbrt_dir):
    from merian_gb300 import scene as S
    return S.load_pbrt(pbrt_dir / "scene.pbrt")


def test_pbrt_geometry_and_instances(native, pbrt_dir):
    from merian_gb300 import _native as N
    sc, cam, (w, h), warnings = _load(pbrt_dir)
    assert (w, h) == (160, 90)
    g = sc.geometries
    # world BLAS: light quad, floor, sphere, ascii ply, disk, measured triangle, textured leaf,
    # checkerboard triangle; then the object
    counts = list(g["triangle_count"])
    assert counts == [2, 2, 64 * 32 * 2, 3, 128, 1, 2, 1, 4]
    assert len(sc.blas_ranges) == 2 and len(sc.instances) == 3
    assert list(sc.blas_ranges["first_geometry"]) == [0, 8]
    assert list(sc.blas_ranges["geometry_count"]) == [8, 1]
    assert list(sc.instances["blas"]) == [0, 1, 1]
    m0 = sc.instances["object_to_world"][0].reshape(3, 4)
    assert np.array_equal(m0, np.eye(3, 4, dtype=np.float32))
    m1 = sc.instances["object_to_world"][1].reshape(3, 4)
    assert np.allclose(m1, [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 3]])
    m2 = sc.instances["object_to_world"][2].reshape(3, 4)
    # Translate(2,0,3) Rotate(90 about y) Scale(0.5): x -> -z / 2, z -> x / 2
    assert np.allclose(m2, [[0, 0, 0.5, 2], [0, 0.5, 0, 0], [-0.5, 0, 0, 3]], atol=1e-6)
    # world-space vertices: the light quad at y = 3, the sphere around (1.5, 0.5, 0)
    pos = sc.vertices["position"]
    v0, n_sph = g["first_vertex"][0], 65 * 33
    assert np.allclose(pos[v0:v0 + 4, 1], 3.0)
    sph = pos[g["first_vertex"][2]:g["first_vertex"][2] + n_sph]
    assert np.allclose(np.linalg.norm(sph - [1.5, 0.5, 0], axis=1), 0.5, atol=1e-5)
    # ply quad fanned into two triangles, mirrored by Scale -1 (FlipFacing), x flipped
    ply = pos[g["first_vertex"][3]:g["first_vertex"][3] + 5]
    assert np.allclose(ply[:, 0], -1.5 - np.array([0, 1, 1, 0, 0.5]))
    assert g["flags"][3] & N.MESH_FLIP_FACING
    assert g["flags"][4] & N.MESH_FLIP_FACING           # ReverseOrientation
    assert not g["flags"][1] & N.MESH_FLIP_FACING
    assert np.all(g["flags"] & N.MESH_TWO_SIDED)
    # object geometry stays in object space (relative to the CTM at ObjectBegin = identity)
    tet = pos[g["first_vertex"][8]:g["first_vertex"][8] + 4]
    assert np.allclose(tet, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    idx = sc.indices
    assert idx.max() < len(sc.vertices)
    assert any("point" in x for x in warnings) and any("checkerboard" in x for x in warnings)
    assert any("measured" in x for x in warnings) and any("curve" in x for x in warnings)


def test_pbrt_materials_camera_env(native, pbrt_dir):
    from merian_gb300 import _native as N
    sc, cam, (w, h), _ = _load(pbrt_dir)
    m = sc.materials[sc.geometries["material_id"]]
    light, floor, sphere, ply, disk, meas, leaf, checks, tree = m
    assert np.allclose(light["emission"], [12, 10.5, 9])
    assert light["model"] == N.MATERIAL_OPENPBR and np.allclose(light["base_color"], 0.5)
    assert np.allclose(light["specular_alpha"], 0.0)   # pbrt's default coated diffuse
    assert np.allclose(floor["base_color"], [0.2, 0.4, 0.6]) and floor["specular_weight"] == 0
    assert sphere["metalness"] == 1 and np.allclose(sphere["base_color"], [1.0, 0.766, 0.336])
    assert np.allclose(sphere["specular_alpha"], math.sqrt(0.04))
    assert ply["model"] == N.MATERIAL_OPENPBR_TRANSMISSION
    assert np.isclose(ply["specular_ior"], 1.33) and ply["transmission_weight"] == 1
    assert disk["metalness"] == 1                       # mix with amount 0.7 -> "gold"
    assert meas["specular_weight"] == 0                 # approximated as diffuse
    assert np.allclose(tree["base_color"], [0.9, 0.8, 0.7])
    assert np.allclose(tree["specular_alpha"], [0.09, 0.16])
    # the imagemap texture: base colour x scale, alpha-tested and two-sided (it has alpha)
    assert leaf["base_color_texture"] == 0 and leaf["alpha_texture"] == 0
    assert np.allclose(leaf["base_color"], 0.8)
    assert sc.geometries["flags"][6] & N.MESH_ALPHA_TEST
    assert len(sc.textures) == 1 and sc.textures[0][1] is True
    assert sc.textures[0][0].shape == (4, 4, 4) and sc.textures[0][0][0, 0, 3] == 0
    assert checks["base_color_texture"] == -1      # checkerboard: unsupported, factor kept
    others = np.delete(m, 6)
    assert np.all(others["base_color_texture"] == -1) and np.all(others["alpha_texture"] == -1)
    # environment: constant L x scale
    assert sc.env is not None and np.allclose(sc.env[..., :3], [0.2, 0.3, 0.4])
    assert sc.env_intensity == 2.0
    # camera: merian's basis from the file's LookAt, fov on the shorter (vertical) axis
    ref = N.Camera()
    lib = N.load()
    P = (N.C.c_float * 3)(0, 1, -5)
    d = np.array([0, -0.5, 5.0]) / np.linalg.norm([0, -0.5, 5.0])
    T = (N.C.c_float * 3)(*(np.array([0, 1, -5]) + d))
    U = (N.C.c_float * 3)(0, 1, 0)
    N.check(lib.gbpt_camera_look_at(P, T, U, math.radians(40), 160 / 90, 0.01, 1000.0,
                                    N.C.byref(ref)))
    for f in ("position", "U", "V", "W"):
        assert np.allclose(np.array(getattr(cam, f)), np.array(getattr(ref, f)), atol=1e-5), f


def test_pbrt_errors(native, tmp_path):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    with pytest.raises(N.GbptError):
        S.load_pbrt(tmp_path / "missing.pbrt")
    (tmp_path / "bad.pbrt").write_text('WorldBegin\nFrobnicate 1 2 3\n')
    with pytest.raises(N.GbptError, match="Frobnicate"):
        S.load_pbrt(tmp_path / "bad.pbrt")
    (tmp_path / "empty.pbrt").write_text('WorldBegin\nLightSource "infinite"\n')
    with pytest.raises(N.GbptError, match="no supported geometry"):
        S.load_pbrt(tmp_path / "empty.pbrt")
    (tmp_path / "unterminated.pbrt").write_text('Shape "trianglemesh "point3 P" [ 0 0 0 ]\n')
    with pytest.raises(N.GbptError):
        S.load_pbrt(tmp_path / "unterminated.pbrt")


def test_pbrt_scene_through_oracle(native, pbrt_dir):
    from merian_gb300 import _native as N
    sc, cam, (w, h), _ = _load(pbrt_dir)
    osc = O.OracleScene(sc)
    hits, _ = osc.trace_primary(cam, w, h, fp64=False, hit_dtype=N.HIT_DTYPE)
    hit = hits["t"] > 0
    assert 0.3 < hit.mean() < 1.0
    # every object is seen: floor, sphere, ply, disk and both tree instances
    seen = set(zip(hits["instance_index"][hit].tolist(), hits["geometry_index"][hit].tolist()))
    assert {(0, 1), (0, 2), (0, 3)} <= seen
    assert any(i in (1, 2) for i, _ in seen)


@pytest.mark.gpu
def test_pbrt_scene_on_gpu(gpu_ctx, pbrt_dir):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc, cam, (w, h), _ = _load(pbrt_dir)
    sid = gpu_ctx.upload(sc)
    try:
        g = gpu_ctx.trace_primary(sid, cam, w, h)
        o, _ = O.OracleScene(sc).trace_primary(cam, w, h, fp64=False, hit_dtype=N.HIT_DTYPE)
        for k in ("instance_id", "instance_index", "geometry_index", "primitive_id"):
            assert np.array_equal(g[k], o[k]), k
        assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
        p, _ = S.render_params(w, h, 64, 6, nee=True, rr_depth=3, frame=2)
        img = gpu_ctx.render(sid, cam, p)
        assert np.all(np.isfinite(img)) and img[:, :3].mean() > 0.05
    finally:
        gpu_ctx.destroy_scene(sid)

"""Alpha-tested (non-opaque) geometry: GBPT_MESH_ALPHA_TEST.

merian runs MaterialSystem::alpha_test on every candidate hit of a non-opaque triangle
(material-system.slang:28-38 from scene.slang:500-519): the material's alpha texture at the
candidate's interpolated uv, alpha below 0.5 discards it. The closest hit is the nearest candidate
that survives; any-hit queries (shadow rays) skip discarded candidates too.

CPU: the oracle on a checkerboard leaf in front of a wall (rays through opaque texels stop at the
leaf, the others reach the wall; without the flag every ray stops at the leaf).
GPU: closest and any hits of incoherent rays on a soup whose alpha textures hold every alpha value
(bilinear filtering crosses 0.5 inside texels) bit-identical to the FP32 oracle, single-level and
instanced; primary hits of the leaf scene bit-identical; its rendered estimate (NEE shadow rays
through the leaf) within 3 sigma of the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import binding as O


def _vertices(pos, uv):
    from merian_gb300 import _native as N
    v = np.zeros(len(pos), N.VERTEX_DTYPE)
    v["position"] = pos
    v["uv"] = np.ascontiguousarray(np.asarray(uv, np.float16)).view(np.uint32).reshape(-1)
    return v


def _material(albedo, alpha_texture=-1):
    from merian_gb300 import _native as N
    m = np.zeros(1, N.MATERIAL_DTYPE)
    m["model"] = N.MATERIAL_DIFFUSE
    m["base_color"] = albedo
    m["base_color_texture"] = -1
    m["alpha_texture"] = alpha_texture
    return m


def leaf_scene(alpha_test=True, cells=8):
    """A wall at z = 1 and, in front of it at z = 0.5, a leaf quad over [0,1]^2 whose uv = (x, y)
    reads a cells x cells alpha checkerboard (opaque where (i + j) is even)."""
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    quad = np.array([[0, 0], [0, 1], [1, 0], [1, 1]], np.float32)
    wall = np.c_[quad * 3 - 1, np.ones(4)].astype(np.float32)
    leaf = np.c_[quad, np.full(4, 0.5)].astype(np.float32)
    verts = np.concatenate([_vertices(wall, quad), _vertices(leaf, quad)])
    idx = np.array([[0, 1, 2], [2, 1, 3]] * 2, np.uint32)
    g = np.zeros(2, N.GEOMETRY_DTYPE)
    g["first_vertex"] = [0, 4]
    g["first_triangle"] = [0, 2]
    g["triangle_count"] = 2
    g["material_id"] = [0, 1]
    base = N.MESH_TWO_SIDED | N.MESH_FLAT_SHADING
    g["flags"] = [base, base | (N.MESH_ALPHA_TEST if alpha_test else 0)]
    g["instance_mask"] = 0xFF
    mats = np.concatenate([_material((0.6, 0.6, 0.6)), _material((0.2, 0.8, 0.2), 0)])
    i, j = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    tex = np.zeros((cells, cells, 4), np.uint8)
    tex[..., :3] = 200
    tex[..., 3] = np.where((i + j) % 2 == 0, 255, 0)
    env = np.ones((8, 16, 4), np.float32)
    return S.SceneData(verts, idx, g, mats, env, textures=[(tex, False)])


def alpha_soup(seed=3, n_geoms=24, tris_per_geom=150, n_tex=5, tex_size=16):
    """Random triangles in the unit cube, half the geometries alpha-tested with random-byte alpha
    textures and random uvs in [-1, 2] (repeat addressing, every alpha value)."""
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    rng = np.random.default_rng(seed)
    n = n_geoms * tris_per_geom
    c = rng.uniform(0, 1, (n, 1, 3))
    pos = (c + rng.normal(0, 0.06, (n, 3, 3))).astype(np.float32).reshape(-1, 3)
    uv = rng.uniform(-1, 2, (3 * n, 2))
    verts = _vertices(pos, uv)
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3) % (3 * tris_per_geom)
    g = np.zeros(n_geoms, N.GEOMETRY_DTYPE)
    g["first_vertex"] = np.arange(n_geoms) * 3 * tris_per_geom
    g["first_triangle"] = np.arange(n_geoms) * tris_per_geom
    g["triangle_count"] = tris_per_geom
    g["material_id"] = np.arange(n_geoms)
    k = np.arange(n_geoms)
    g["flags"] = (np.where(k % 2 == 0, N.MESH_ALPHA_TEST, 0) |
                  np.where(k % 3 == 0, N.MESH_TWO_SIDED, 0)).astype(np.uint32)
    g["instance_mask"] = 0xFF
    mats = np.concatenate([_material(rng.uniform(0.2, 0.8, 3), int(k % n_tex) if k % 4 else -1)
                           for k in range(n_geoms)])
    textures = [(rng.integers(0, 256, (tex_size, tex_size, 4), dtype=np.uint8), bool(t % 2))
                for t in range(n_tex)]
    return S.SceneData(verts, idx, g, mats, None, textures=textures)


def instanced(sc, n_inst=6, seed=4):
    """The soup as one BLAS placed n_inst times (rotations, scales 0.5-2, offsets in a 4^3 box)."""
    from merian_gb300 import _native as N
    rng = np.random.default_rng(seed)
    blas = np.zeros(1, N.BLAS_DTYPE)
    blas["first_geometry"] = 0
    blas["geometry_count"] = len(sc.geometries)
    inst = np.zeros(n_inst, N.INSTANCE_DTYPE)
    for k in range(n_inst):
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        m = np.c_[q * rng.uniform(0.5, 2.0), rng.uniform(0, 4, 3)]
        inst[k]["object_to_world"] = m.astype(np.float32).reshape(-1)
        inst[k]["mask"] = 0xFF
    from merian_gb300 import scene as S
    return S.SceneData(sc.vertices, sc.indices, sc.geometries, sc.materials, None,
                       blas_ranges=blas, instances=inst, textures=sc.textures)


def random_rays(n, seed, lo=-0.2, hi=1.2):
    from merian_gb300 import _native as N
    rng = np.random.default_rng(seed)
    r = np.zeros(n, N.RAY_DTYPE)
    r["origin"] = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    r["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r["tmax"] = 1e7
    return r


def _z_rays(cells=8):
    """One +z ray through every texel centre of the leaf."""
    from merian_gb300 import _native as N
    xs = (np.arange(cells) + 0.5) / cells
    x, y = np.meshgrid(xs, xs, indexing="ij")
    r = np.zeros(cells * cells, N.RAY_DTYPE)
    r["origin"] = np.c_[x.reshape(-1), y.reshape(-1), np.zeros(cells * cells)]
    r["direction"] = (0, 0, 1)
    r["tmax"] = 1e7
    return r, ((np.arange(cells)[:, None] + np.arange(cells)[None, :]) % 2 == 0).reshape(-1)


def test_oracle_alpha_checkerboard(native):
    from merian_gb300 import _native as N
    rays, opaque = _z_rays()
    for fp64 in (False, True):
        h, _, _ = O.OracleScene(leaf_scene(True)).trace_rays(rays, fp64=fp64, hit_dtype=N.HIT_DTYPE)
        assert np.array_equal(h["geometry_index"] == 1, opaque)
        assert np.allclose(h["t"], np.where(opaque, 0.5, 1.0))
        a, _, _ = O.OracleScene(leaf_scene(True)).trace_rays(rays, fp64=fp64, any_hit=True,
                                                              hit_dtype=N.HIT_DTYPE)
        assert np.all(a["t"] > 0)  # the wall stops the transparent ones
    h, _, _ = O.OracleScene(leaf_scene(False)).trace_rays(rays, hit_dtype=N.HIT_DTYPE)
    assert np.all(h["geometry_index"] == 1)


def test_oracle_alpha_soup_discards(native):
    """Alpha-tested geometry loses hits to the geometry behind it; opaque copies do not."""
    from merian_gb300 import _native as N
    sc = alpha_soup()
    rays = random_rays(4000, 1)
    a, _, _ = O.OracleScene(sc).trace_rays(rays, hit_dtype=N.HIT_DTYPE)
    opaque = alpha_soup()
    opaque.geometries["flags"] &= ~np.uint32(N.MESH_ALPHA_TEST)
    b, _, _ = O.OracleScene(opaque).trace_rays(rays, hit_dtype=N.HIT_DTYPE)
    diff = (a["geometry_index"] != b["geometry_index"]) | (a["primitive_id"] != b["primitive_id"])
    assert 0.02 < diff.mean() < 0.6
    # a discarded opaque-scene hit lies on an alpha-tested geometry, and the new hit is farther
    hit_b = b["t"] > 0
    moved = diff & hit_b
    assert np.all(sc.geometries["flags"][b["geometry_index"][moved]] & N.MESH_ALPHA_TEST)
    later = a["t"][moved]
    assert np.all((later < 0) | (later >= b["t"][moved]))


@pytest.fixture(scope="module")
def alpha_scenes(gpu_ctx):
    soup = alpha_soup()
    inst = instanced(soup)
    leaf = leaf_scene(True)
    ids = [gpu_ctx.upload(s) for s in (soup, inst, leaf)]
    yield list(zip((soup, inst, leaf), ids))
    for sid in ids:
        gpu_ctx.destroy_scene(sid)


def _gpu_trace(gpu_ctx, sid, rays, any_hit=False):
    import torch
    from merian_gb300 import _native as N
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(rays) * N.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr(), any_hit=any_hit)
    gpu_ctx.synchronize()
    return d_hits.cpu().numpy().view(N.HIT_DTYPE)


@pytest.mark.gpu
@pytest.mark.parametrize("which", [0, 1])
def test_alpha_rays_bit_exact(gpu_ctx, alpha_scenes, which):
    from merian_gb300 import _native as N
    sc, sid = alpha_scenes[which]
    rays = random_rays(200_000, 7, hi=1.2 if which == 0 else 5.0)
    g = _gpu_trace(gpu_ctx, sid, rays)
    o, _, _ = O.OracleScene(sc).trace_rays(rays, fp64=False, hit_dtype=N.HIT_DTYPE)
    assert (o["t"] > 0).mean() > 0.2
    for k in ("instance_id", "instance_index", "geometry_index", "primitive_id"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
    assert np.array_equal(g["barycentrics"].view(np.uint32), o["barycentrics"].view(np.uint32))
    ga = _gpu_trace(gpu_ctx, sid, rays, any_hit=True)
    oa, _, _ = O.OracleScene(sc).trace_rays(rays, fp64=False, any_hit=True, hit_dtype=N.HIT_DTYPE)
    assert np.array_equal(ga["t"] > 0, oa["t"] > 0)
    assert np.array_equal(ga["t"] > 0, o["t"] > 0)


@pytest.mark.gpu
def test_alpha_leaf_primary_and_render(gpu_ctx, alpha_scenes):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc, sid = alpha_scenes[2]
    osc = O.OracleScene(sc)
    cam = S.look_at((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), (0, 1, 0), 50.0, 1.0)
    g = gpu_ctx.trace_primary(sid, cam, 96, 96)
    o, _ = osc.trace_primary(cam, 96, 96, fp64=False, hit_dtype=N.HIT_DTYPE)
    for k in ("geometry_index", "primitive_id"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
    leaf = g["geometry_index"] == 1
    assert 0.2 < leaf.mean() < 0.6  # half the leaf's texels are holes
    rng = np.random.default_rng(5)
    pix = np.sort(rng.choice(96 * 96, 48, replace=False)).astype(np.uint32)
    spp = 4096
    p, k1 = S.render_params(96, 96, spp, 5, nee=True, rr_depth=3, frame=1, pixels=pix)
    gm = gpu_ctx.render(sid, cam, p)[:, :3].astype(np.float64)
    p2, k2 = S.render_params(96, 96, spp, 5, nee=True, rr_depth=3, frame=77, pixels=pix)
    om, osq, _ = osc.render(cam, p2, fp64=True)
    om = om[:, :3]
    var = np.maximum(osq - om * om, 0.0)
    se = np.sqrt(2 * var / spp) + 1e-5 * np.abs(om) + 1e-7
    z = (gm - om) / se
    assert np.mean(np.abs(z) > 3) <= 0.03 and np.mean(z * z) < 1.6
    # the wall behind a hole is lit through the leaf's holes: brighter than behind opaque texels
    opaque_scene = leaf_scene(False)
    sid2 = gpu_ctx.upload(opaque_scene)
    try:
        full, _ = S.render_params(96, 96, 64, 5, nee=True, rr_depth=3, frame=3)
        a = gpu_ctx.render(sid, cam, full)[:, :3].mean()
        b = gpu_ctx.render(sid2, cam, full)[:, :3].mean()
        assert a != b
    finally:
        gpu_ctx.destroy_scene(sid2)


@pytest.mark.gpu
def test_alpha_batch_equals_alone(gpu_ctx, alpha_scenes):
    """A tick that holds an alpha-tested scene runs the alpha-test traversal variants for every
    request in it; requests on opaque scenes still give the same bits as alone."""
    from merian_gb300 import scene as S
    corn = gpu_ctx.upload(S.cornell())
    try:
        (soup, sid_soup), (_, sid_inst), (leaf, sid_leaf) = alpha_scenes
        cam_c = S.workload_camera("cornell-256-16spp")
        cam_l = S.look_at((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), (0, 1, 0), 50.0, 1.0)
        cam_s = S.look_at((0.5, 0.5, -0.8), (0.5, 0.5, 0.5), (0, 1, 0), 50.0, 1.0)
        jobs = []
        for i, (sid, cam) in enumerate([(corn, cam_c), (sid_leaf, cam_l), (sid_soup, cam_s),
                                        (sid_inst, cam_s)]):
            p, _ = S.render_params(64, 64, 8, 5, nee=True, rr_depth=3, frame=40 + i)
            jobs.append((sid, cam, p))
        alone = [gpu_ctx.render(*j) for j in jobs]
        outs = gpu_ctx.render_batch(jobs)
        for a, b in zip(alone, outs):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    finally:
        gpu_ctx.destroy_scene(corn)

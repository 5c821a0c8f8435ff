"""Two-level (instanced) scenes and textures.

CPU: the oracle's instanced traversal against the same scene flattened into world space (the
instance transforms applied to the vertices in double): same closest hits except where the two
float roundings of a vertex differ (at most 0.2 % of the rays), t within 1e-4 relative.
GPU: the library against the FP32 oracle on the instanced scene: primary hits and incoherent rays
bit-identical (the object-space ray is formed with the same rounded operations on both sides);
GBuffer texels (textured albedo) to FP32 round-off; the rendered estimate within 3 sigma of the
FP64 oracle.
"""
import numpy as np
import pytest

from oracle import binding as O


def small_instanced(seed=5):
    from merian_gb300 import workloads as W
    return W.instanced_scene(seed, n_meshes=4, n_u=60, n_v=31, n_instances=60, n_textures=6,
                             tex_size=64, bands=3, box=20.0, env_size=(128, 64))


def flatten(sc):
    """The same scene as one level: every instance's copy of its BLAS in world space."""
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    verts, idx, geoms = [], [], []
    v_off = t_off = 0
    for inst in sc.instances:
        M = inst["object_to_world"].astype(np.float64).reshape(3, 4)
        r = sc.blas_ranges[inst["blas"]]
        for gi in range(r["first_geometry"], r["first_geometry"] + r["geometry_count"]):
            g = sc.geometries[gi].copy()
            tri = sc.indices[g["first_triangle"]:g["first_triangle"] + g["triangle_count"]]
            vi = np.unique(tri) + g["first_vertex"]
            remap = {int(v): k for k, v in enumerate(vi)}
            v = sc.vertices[vi].copy()
            p = v["position"].astype(np.float64)
            v["position"] = (p @ M[:, :3].T + M[:, 3]).astype(np.float32)
            t = np.vectorize(lambda x: remap[int(x) + int(g["first_vertex"])])(tri).astype(np.uint32)
            g["first_vertex"] = v_off
            g["first_triangle"] = t_off
            verts.append(v)
            idx.append(t)
            geoms.append(g)
            v_off += len(v)
            t_off += len(t)
    return S.SceneData(np.concatenate(verts), np.concatenate(idx),
                       np.array(geoms, dtype=N.GEOMETRY_DTYPE), sc.materials, sc.env)


def random_rays(n, seed, box=20.0):
    from merian_gb300 import _native as N
    rng = np.random.default_rng(seed)
    r = np.zeros(n, N.RAY_DTYPE)
    r["origin"] = rng.uniform(-0.2 * box, 1.2 * box, size=(n, 3))
    d = rng.normal(size=(n, 3))
    r["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r["tmin"] = 0.0
    r["tmax"] = 1e7
    return r


def test_oracle_instancing_matches_flattened_scene(native):
    from merian_gb300 import _native as N
    sc = small_instanced()
    inst = O.OracleScene(sc)
    flat = O.OracleScene(flatten(sc))
    rays = random_rays(20_000, 3)
    a, _, _ = inst.trace_rays(rays, fp64=False, hit_dtype=N.HIT_DTYPE)
    b, _, _ = flat.trace_rays(rays, fp64=False, hit_dtype=N.HIT_DTYPE)
    hit_a, hit_b = a["t"] > 0, b["t"] > 0
    assert hit_a.mean() > 0.05
    assert np.mean(hit_a != hit_b) < 2e-3
    both = hit_a & hit_b
    # the flattened geometry index enumerates (instance, BLAS geometry) pairs in order
    first = sc.blas_ranges["first_geometry"][sc.instances["blas"]]
    cnt = sc.blas_ranges["geometry_count"][sc.instances["blas"]]
    flat_base = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    g_expect = flat_base[a["instance_index"][both]] + a["geometry_index"][both]
    same = (g_expect == b["geometry_index"][both]) & (a["primitive_id"][both] == b["primitive_id"][both])
    assert same.mean() > 0.998
    assert np.all(a["instance_id"][both] == first[a["instance_index"][both]])
    rel = np.abs(a["t"][both].astype(np.float64) - b["t"][both]) / b["t"][both]
    # FP32 object-space rays (origins up to ~30 units away, scales up to 2): t agrees to a few
    # ulps of the transformed origin
    assert np.median(rel) < 1e-6 and np.mean(rel < 1e-4) > 0.998


@pytest.fixture(scope="module")
def inst_scene(gpu_ctx):
    from merian_gb300 import workloads as W
    sc = small_instanced()
    sid = gpu_ctx.upload(sc)
    yield sc, sid, O.OracleScene(sc), W.instanced_camera(160, 90, box=20.0)
    gpu_ctx.destroy_scene(sid)


@pytest.mark.gpu
def test_instanced_primary_hits_bit_exact(gpu_ctx, inst_scene):
    from merian_gb300 import _native as N
    sc, sid, osc, cam = inst_scene
    g = gpu_ctx.trace_primary(sid, cam, 160, 90)
    o, _ = osc.trace_primary(cam, 160, 90, fp64=False, hit_dtype=N.HIT_DTYPE)
    assert (g["t"] > 0).mean() > 0.2
    for k in ("instance_id", "instance_index", "geometry_index", "primitive_id"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
    assert np.array_equal(g["barycentrics"].view(np.uint32), o["barycentrics"].view(np.uint32))


@pytest.mark.gpu
def test_instanced_rays_bit_exact(gpu_ctx, inst_scene):
    import torch
    from merian_gb300 import _native as N
    sc, sid, osc, cam = inst_scene
    rays = random_rays(100_000, 9)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(rays) * N.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr())
    gpu_ctx.synchronize()
    g = d_hits.cpu().numpy().view(N.HIT_DTYPE)
    o, _, _ = osc.trace_rays(rays, fp64=False, hit_dtype=N.HIT_DTYPE)
    for k in ("instance_index", "geometry_index", "primitive_id"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
    gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr(), any_hit=True)
    gpu_ctx.synchronize()
    ga = d_hits.cpu().numpy().view(N.HIT_DTYPE)
    assert np.array_equal(ga["t"] > 0, o["t"] > 0)


@pytest.mark.gpu
def test_instanced_gbuffer_textured_albedo(gpu_ctx, inst_scene):
    import ctypes as C
    import torch
    from merian_gb300 import _native as N
    sc, sid, osc, cam = inst_scene
    buf = torch.zeros(160 * 90 * 16, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    N.check(gpu_ctx.lib.gbpt_gbuffer(gpu_ctx.handle, sid, C.byref(cam), 160, 90, 0xFF,
                                     buf.data_ptr()))
    gpu_ctx.synchronize()
    g = buf.cpu().numpy().view(N.GBUFFER_DTYPE)
    o = osc.gbuffer(cam, 160, 90, texel_dtype=N.GBUFFER_DTYPE)
    for k in ("instance_id", "instance_index", "geometry_index", "primitive_id", "barycentrics"):
        assert np.array_equal(g[k], o[k]), k
    assert np.allclose(g["albedo"], o["albedo"], rtol=1e-4, atol=1e-6)
    hit = g["instance_id"] != 0xFFFFFFFF
    # textured: the albedo varies within a geometry
    gi = g["geometry_index"][hit].astype(np.int64) + g["instance_id"][hit]
    a = g["albedo"][hit][:, 0]
    assert any(np.ptp(a[gi == k]) > 0.05 for k in np.unique(gi))


@pytest.mark.gpu
def test_instanced_render_converges_to_oracle(gpu_ctx, inst_scene):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc, sid, osc, cam = inst_scene
    hits = gpu_ctx.trace_primary(sid, cam, 160, 90)
    rng = np.random.default_rng(2)
    on = np.flatnonzero(hits["t"] > 0)
    pix = np.sort(np.concatenate([rng.choice(on, 40, replace=False),
                                  rng.choice(np.flatnonzero(hits["t"] <= 0), 8, replace=False)]))
    pix = pix.astype(np.uint32)
    spp = 4096
    p, k1 = S.render_params(160, 90, spp, 8, nee=True, rr_depth=3, frame=1, pixels=pix)
    gm = gpu_ctx.render(sid, cam, p)[:, :3].astype(np.float64)
    p2, k2 = S.render_params(160, 90, spp, 8, nee=True, rr_depth=3, frame=99, pixels=pix)
    om, osq, _ = osc.render(cam, p2, fp64=True)
    om = om[:, :3]
    var = np.maximum(osq - om * om, 0.0)
    se = np.sqrt(2 * var / spp) + 1e-5 * np.abs(om) + 1e-7
    z = (gm - om) / se
    assert np.mean(np.abs(z) > 3) <= 0.03 and np.mean(z * z) < 1.6

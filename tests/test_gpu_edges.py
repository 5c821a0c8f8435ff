"""Edge cases of the render path: a scene with no geometry (environment only), a scene of one
triangle, one pixel with many samples in one tick, and a frame larger than one tick (33.5 M
paths) whose pixels must equal the same pixels rendered as a list.

CPU: the oracle on the empty scene (every ray misses).
GPU: bit-exact primary hits on the one-triangle scene; radiance within 4 sigma of the FP64
oracle; subset consistency across tick boundaries.
"""
import numpy as np
import pytest

from oracle import binding as O


def env_only():
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    h, w = 16, 32
    v, u = np.meshgrid(np.linspace(0, 1, h), np.linspace(0, 1, w), indexing="ij")
    env = np.stack([0.2 + u, 0.5 + 0 * u, 0.2 + v, np.ones_like(u)], -1).astype(np.float32)
    m = np.zeros(1, N.MATERIAL_DTYPE)
    m["base_color_texture"] = -1
    m["alpha_texture"] = -1
    return S.SceneData(np.zeros(0, N.VERTEX_DTYPE), np.zeros((0, 3), np.uint32),
                       np.zeros(0, N.GEOMETRY_DTYPE), m, env)


def one_triangle():
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    v = np.zeros(3, N.VERTEX_DTYPE)
    v["position"] = [[-1, -1, 2], [1, -1, 2], [0, 1, 2]]
    g = np.zeros(1, N.GEOMETRY_DTYPE)
    g["triangle_count"] = 1
    g["flags"] = N.MESH_TWO_SIDED | N.MESH_FLAT_SHADING
    g["instance_mask"] = 0xFF
    m = np.zeros(1, N.MATERIAL_DTYPE)
    m["model"] = N.MATERIAL_OPENPBR
    m["base_color"] = 0.5
    m["specular_alpha"] = 0.3
    m["specular_weight"] = 1.0
    m["specular_ior"] = 1.5
    m["emission"] = [1.0, 2.0, 3.0]
    m["base_color_texture"] = -1
    m["alpha_texture"] = -1
    env = np.full((8, 16, 4), 0.5, np.float32)
    return S.SceneData(v, np.array([[0, 1, 2]], np.uint32), g, m, env)


def _z(gm, om, osq, spp):
    var = np.maximum(osq - om * om, 0.0)
    se = np.sqrt(2 * var / spp) + 1e-5 * np.abs(om) + 1e-7
    return (gm - om) / se


def test_oracle_empty_scene_misses(native):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc = env_only()
    cam = S.look_at((0, 0, 0), (0, 0, 1), (0, 1, 0), 60.0, 2.0)
    hits, _ = O.OracleScene(sc).trace_primary(cam, 32, 16, fp64=False, hit_dtype=N.HIT_DTYPE)
    assert np.all(hits["t"] < 0) and np.all(hits["instance_id"] == 0xFFFFFFFF)


@pytest.mark.gpu
def test_env_only_scene_matches_oracle(gpu_ctx):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc = env_only()
    sid = gpu_ctx.upload(sc)
    try:
        cam = S.look_at((0, 0, 0), (0, 0, 1), (0, 1, 0), 60.0, 2.0)
        g = gpu_ctx.trace_primary(sid, cam, 32, 16)
        assert np.all(g["t"] < 0) and np.all(g["instance_id"] == 0xFFFFFFFF)
        for nee in (False, True):
            p, _ = S.render_params(32, 16, 256, 5, nee=nee, frame=3)
            gm = gpu_ctx.render(sid, cam, p)[:, :3].astype(np.float64)
            p2, _ = S.render_params(32, 16, 256, 5, nee=nee, frame=9)
            om, osq, _ = O.OracleScene(sc).render(cam, p2, fp64=True)
            z = _z(gm, om[:, :3], osq, 256)
            assert np.mean(np.abs(z) > 4) <= 0.01 and np.mean(z * z) < 1.6
    finally:
        gpu_ctx.destroy_scene(sid)


@pytest.mark.gpu
def test_one_triangle_scene(gpu_ctx):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc = one_triangle()
    sid = gpu_ctx.upload(sc)
    osc = O.OracleScene(sc)
    try:
        cam = S.look_at((0, 0, 0), (0, 0, 1), (0, 1, 0), 70.0, 1.0)
        g = gpu_ctx.trace_primary(sid, cam, 64, 64)
        o, _ = osc.trace_primary(cam, 64, 64, fp64=False, hit_dtype=N.HIT_DTYPE)
        assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
        assert np.array_equal(g["barycentrics"].view(np.uint32), o["barycentrics"].view(np.uint32))
        assert 0.2 < (g["t"] > 0).mean() < 0.8
        rng = np.random.default_rng(1)
        pix = np.sort(rng.choice(64 * 64, 64, replace=False)).astype(np.uint32)
        p, k1 = S.render_params(64, 64, 2048, 6, nee=True, rr_depth=3, frame=5, pixels=pix)
        gm = gpu_ctx.render(sid, cam, p)[:, :3].astype(np.float64)
        p2, k2 = S.render_params(64, 64, 2048, 6, nee=True, rr_depth=3, frame=6, pixels=pix)
        om, osq, _ = osc.render(cam, p2, fp64=True)
        z = _z(gm, om[:, :3], osq, 2048)
        assert np.mean(np.abs(z) > 4) <= 0.02 and np.mean(z * z) < 1.6
    finally:
        gpu_ctx.destroy_scene(sid)


@pytest.mark.gpu
def test_one_pixel_many_samples(gpu_ctx):
    from merian_gb300 import scene as S
    sc = one_triangle()
    sid = gpu_ctx.upload(sc)
    try:
        cam = S.look_at((0, 0, 0), (0, 0, 1), (0, 1, 0), 10.0, 1.0)
        spp = 200_000
        p, _ = S.render_params(1, 1, spp, 6, nee=True, rr_depth=3, frame=1)
        gm = gpu_ctx.render(sid, cam, p)[:, :3].astype(np.float64)
        p2, _ = S.render_params(1, 1, 65536, 6, nee=True, rr_depth=3, frame=2)
        om, osq, _ = O.OracleScene(sc).render(cam, p2, fp64=True)
        var = np.maximum(osq - om[:, :3] ** 2, 0.0)
        se = np.sqrt(var / spp + var / 65536) + 1e-6
        assert np.all(np.abs(gm - om[:, :3]) < 5 * se)
    finally:
        gpu_ctx.destroy_scene(sid)


@pytest.mark.gpu
def test_frame_larger_than_a_tick_matches_pixel_list(gpu_ctx):
    """8192 x 4096 x 1 spp = 33.5 M paths: several ticks; any pixel equals the same pixel
    rendered alone from a pixel list, bit for bit."""
    import torch
    from merian_gb300 import scene as S
    sc = one_triangle()
    sid = gpu_ctx.upload(sc)
    try:
        W, H = 8192, 4096
        cam = S.look_at((0, 0, 0), (0, 0, 1), (0, 1, 0), 70.0, W / H)
        out = torch.empty((W * H, 4), device="cuda")
        p, _ = S.render_params(W, H, 1, 4, nee=True, rr_depth=3, frame=11)
        gpu_ctx.render_device(sid, cam, p, out.data_ptr())
        gpu_ctx.synchronize()
        rng = np.random.default_rng(3)
        pix = np.sort(np.concatenate([rng.choice(W * H, 2000, replace=False),
                                      [0, W - 1, W * H - 1, (1 << 24) - 1, 1 << 24]]))
        pix = np.unique(pix).astype(np.uint32)
        pl, keep = S.render_params(W, H, 1, 4, nee=True, rr_depth=3, frame=11, pixels=pix)
        sub = gpu_ctx.render(sid, cam, pl)
        full = out[torch.from_numpy(pix.astype(np.int64)).cuda()].cpu().numpy()
        assert np.array_equal(full.view(np.uint32), sub.view(np.uint32))
    finally:
        gpu_ctx.destroy_scene(sid)


@pytest.mark.gpu
def test_bvh_build_modes_find_the_same_hits(gpu_ctx):
    """GBPT_BVH_SPLIT (default), _MEDIUM and _FAST build different trees (split references or
    not); closest and any hits of incoherent rays are the same bits in all three, and equal the
    FP32 oracle's."""
    import torch
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc = S.soup(S.BASE_SEED, 100_000, 64, (64, 32))
    rng = np.random.default_rng(2)
    rays = np.zeros(100_000, N.RAY_DTYPE)
    rays["origin"] = rng.uniform(-0.2, 1.2, (len(rays), 3))
    d = rng.normal(size=(len(rays), 3))
    rays["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmax"] = 1e7
    o, _, _ = O.OracleScene(sc).trace_rays(rays, fp64=False, hit_dtype=N.HIT_DTYPE)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(rays) * N.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    nodes = []
    try:
        for mode in (N.BVH_FAST, N.BVH_MEDIUM, N.BVH_SPLIT):
            gpu_ctx.set_tuning(bvh_build=mode)
            sid = gpu_ctx.upload(sc)
            try:
                nodes.append(gpu_ctx.scene_stats(sid)["nodes"])
                for any_hit in (False, True):
                    gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr(),
                                  any_hit=any_hit)
                    gpu_ctx.synchronize()
                    g = d_hits.cpu().numpy().view(N.HIT_DTYPE)
                    if any_hit:
                        assert np.array_equal(g["t"] > 0, o["t"] > 0)
                    else:
                        assert np.array_equal(g["primitive_id"], o["primitive_id"])
                        assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
            finally:
                gpu_ctx.destroy_scene(sid)
        assert nodes[0] < nodes[1] < nodes[2]
    finally:
        gpu_ctx.set_tuning()


@pytest.mark.gpu
@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_facing_per_axis_matches_oracle(gpu_ctx, axis, sign):
    """The kernels read each triangle in the order of the ray's dominant axis from one of three
    stored copies and flip the facing for a negative direction: one-sided, reversed, FlipFacing
    and TwoSided triangles seen along each axis both ways give the oracle's hits and bits."""
    import torch
    from conftest import facing_case
    from merian_gb300 import _native as N
    sc, rays, expect, t_expect = facing_case(axis, sign)
    osc = O.OracleScene(sc)
    sid = gpu_ctx.upload(sc)
    try:
        d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
        d_hits = torch.zeros(len(rays) * N.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        for mask, hit in expect.items():
            for any_hit in (False, True):
                gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr(), mask=mask,
                              any_hit=any_hit)
                gpu_ctx.synchronize()
                g = d_hits.cpu().numpy().view(N.HIT_DTYPE)
                assert (g["geometry_index"][0] != 0xFFFFFFFF) == hit, (mask, any_hit)
            o, _, _ = osc.trace_rays(rays, mask=mask, hit_dtype=N.HIT_DTYPE)
            assert g["geometry_index"][0] == o["geometry_index"][0]
            if hit:
                assert g["t"].view(np.uint32)[0] == o["t"].view(np.uint32)[0]
    finally:
        gpu_ctx.destroy_scene(sid)

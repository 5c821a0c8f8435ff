"""The CWBVH the package builds, walked on the host.

CPU: gbpt_bvh_build gives the tree gbpt_scene_create uploads, deterministically and the same on
every host (a fixed partition of the parallel build); the oracle's walk of that tree
(oracle_cwbvh_trace, the device traversal order restated) finds exactly the FP32 oracle's hits
(its own binary BVH) for incoherent rays, closest and any hit.
GPU: the device traversal without postponed triangle groups (trace_postpone_lanes = 1) visits
exactly the nodes and tests exactly the triangles the walk does, and returns the same hits: the
walk's counts are the roofline's per-ray figures, pinned to the kernel's own counters.
"""
import hashlib

import numpy as np
import pytest

from oracle import binding as O

# sha256 prefix of the soup_small tree (nodes then triangle records), whatever the host
SOUP_SMALL_BVH = "e7c987c5f2a72ad1"


def _soup_small():
    from merian_gb300 import scene as S
    return S.soup(S.BASE_SEED, 200_000, 256, (256, 128))


def _rays(n, seed):
    from merian_gb300 import _native as N
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, N.RAY_DTYPE)
    rays["origin"] = rng.uniform(-0.1, 1.1, size=(n, 3))
    d = rng.normal(size=(n, 3))
    rays["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmax"] = np.where(rng.uniform(size=n) < 0.2, rng.uniform(0.01, 0.5, size=n), 1e7)
    return rays


def _same_hits(a, b):
    return (np.array_equal(a["geometry_index"], b["geometry_index"]) and
            np.array_equal(a["primitive_id"], b["primitive_id"]) and
            np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32)) and
            np.array_equal(a["barycentrics"].view(np.uint32), b["barycentrics"].view(np.uint32)))


def test_host_build_is_deterministic_and_host_independent(native):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc = _soup_small()
    n1, t1, d1 = S.build_bvh(sc)
    n2, t2, d2 = S.build_bvh(sc)
    assert np.array_equal(n1, n2) and np.array_equal(t1, t2) and d1 == d2
    assert 0 < d1 <= 24 and len(t1) >= sc.triangle_count
    assert hashlib.sha256(n1.tobytes() + t1.tobytes()).hexdigest()[:16] == SOUP_SMALL_BVH
    # one reference per triangle without split clipping
    _, tf, _ = S.build_bvh(sc, N.BVH_FAST)
    assert len(tf) == sc.triangle_count


@pytest.mark.parametrize("which", ["cornell", "soup_small"])
def test_walk_matches_oracle_hits(native, which):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc = S.cornell() if which == "cornell" else _soup_small()
    nodes, tris, _ = S.build_bvh(sc)
    rays = _rays(100_000, 3)
    osc = O.OracleScene(sc)
    for any_hit in (False, True):
        w, counts = O.cwbvh_trace(nodes, tris, rays, any_hit=any_hit, hit_dtype=N.HIT_DTYPE)
        o, _, _ = osc.trace_rays(rays, fp64=False, any_hit=any_hit, hit_dtype=N.HIT_DTYPE)
        if any_hit:
            assert np.array_equal(w["geometry_index"] != 0xFFFFFFFF,
                                  o["geometry_index"] != 0xFFFFFFFF)
        else:
            assert _same_hits(w, o)
        assert counts[:, 0].min() >= 1 and counts.sum() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("any_hit", [False, True], ids=["closest", "any"])
def test_kernel_counts_match_host_walk(gpu_ctx, any_hit):
    import torch
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    sc = _soup_small()
    nodes, tris, _ = S.build_bvh(sc)
    sid = gpu_ctx.upload(sc)
    rays = _rays(200_000, 17)
    try:
        gpu_ctx.set_tuning(0, -1, False, postpone_lanes=1)
        d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
        d_hits = torch.zeros(len(rays) * N.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        npr, tpr = gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr(),
                                 any_hit=any_hit, counted=True)
        gpu_ctx.synchronize()
        g = d_hits.cpu().numpy().view(N.HIT_DTYPE)
        w, counts = O.cwbvh_trace(nodes, tris, rays, any_hit=any_hit, hit_dtype=N.HIT_DTYPE)
        assert round(npr * len(rays)) == int(counts[:, 0].sum())
        assert round(tpr * len(rays)) == int(counts[:, 1].sum())
        if any_hit:
            assert np.array_equal(g["geometry_index"] != 0xFFFFFFFF,
                                  w["geometry_index"] != 0xFFFFFFFF)
        else:
            assert _same_hits(g, w)
    finally:
        gpu_ctx.set_tuning(0, -1, False)
        gpu_ctx.destroy_scene(sid)

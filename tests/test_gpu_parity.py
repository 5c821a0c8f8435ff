"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances:
  * primary hits vs the FP32 oracle: identical (geometry, primitive) ids and bit-identical t (the
    camera ray and the watertight test are computed with the same IEEE operations on both sides);
  * primary hits vs the FP64 oracle: t within 1e-5 relative; ids may differ only at ties, where
    the FP64 distance to both candidates agrees within 1e-5 relative;
  * per-pixel mean radiance vs the FP64 oracle fixture: |z| > 3 on at most 2% of the channels and
    mean z^2 < 1.5 (z = difference over the combined standard error of both estimators, floored
    at 1e-5 relative for FP32 round-off); the relative RMSE must be explained by that noise
    (at most 1.25x the noise RMSE);
  * the output's `a` channel (mean squared YUV luminance, render_pt.slang:110-129) vs the
    fixture's, by the same z test, for the BSDF-only estimator: the fixtures hold the reference's
    BSDF-only estimator, and a second moment, unlike the mean, depends on the estimator (NEE and
    roulette change the distribution of the samples, not their expectation).
The relative RMSE against the fixture is printed per configuration and estimator.
"""
import numpy as np
import pytest

from conftest import ROOT
from oracle import binding as O

pytestmark = pytest.mark.gpu


def golden(name):
    return np.load(ROOT / "tests" / "golden" / f"{name}.npz")


def _check_scene_hash(sc, name):
    """The fixture was computed on this exact scene (the generators are host-independent)."""
    import sys
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from make_golden import scene_hash
    assert scene_hash(sc) == str(golden(name)["scene_hash"]), f"{name}: scene differs from fixture"


@pytest.fixture(scope="module")
def cornell(gpu_ctx):
    from merian_gb300 import scene as S
    sc = S.cornell()
    _check_scene_hash(sc, "cornell")
    sid = gpu_ctx.upload(sc)
    yield sc, sid, O.OracleScene(sc), S.workload_camera("cornell-256-16spp")
    gpu_ctx.destroy_scene(sid)


@pytest.fixture(scope="module")
def soup_1m(gpu_ctx):
    """The benchmarked 1M-triangle soup with its 2048x1024 environment and the 1080p camera."""
    from merian_gb300 import scene as S
    sc = S.workload_scene("soup-1m-1080p-64spp")
    _check_scene_hash(sc, "soup_1m")
    sid = gpu_ctx.upload(sc)
    yield sc, sid, None, S.workload_camera("soup-1m-1080p-64spp")
    gpu_ctx.destroy_scene(sid)


@pytest.fixture(scope="module")
def soup_small(gpu_ctx):
    from merian_gb300 import scene as S
    sc = S.soup(S.BASE_SEED, 200_000, 256, (256, 128))
    _check_scene_hash(sc, "soup_small")
    sid = gpu_ctx.upload(sc)
    cam = S.look_at((0.5, 0.5, -1.2), (0.5, 0.5, 0.5), (0, 1, 0), 45.0, 16 / 9)
    yield sc, sid, O.OracleScene(sc), cam
    gpu_ctx.destroy_scene(sid)


def _primary_checks(gpu_ctx, sid, osc, cam, w, h):
    from merian_gb300 import _native as N
    g = gpu_ctx.trace_primary(sid, cam, w, h)
    o32, _ = osc.trace_primary(cam, w, h, fp64=False, hit_dtype=N.HIT_DTYPE)
    # FP32 oracle: exact
    assert np.array_equal(g["geometry_index"], o32["geometry_index"])
    assert np.array_equal(g["primitive_id"], o32["primitive_id"])
    assert np.array_equal(g["t"].view(np.uint32), o32["t"].view(np.uint32))
    assert np.array_equal(g["barycentrics"].view(np.uint32), o32["barycentrics"].view(np.uint32))
    # FP64 oracle: t within 1e-5, id mismatches only at ties
    o64, t64 = osc.trace_primary(cam, w, h, fp64=True, hit_dtype=N.HIT_DTYPE)
    hit = g["t"] > 0
    assert np.array_equal(hit, t64 > 0)
    rel = np.abs(g["t"][hit].astype(np.float64) - t64[hit]) / t64[hit]
    assert rel.max() < 1e-5
    diff = hit & ((g["geometry_index"] != o64["geometry_index"]) |
                  (g["primitive_id"] != o64["primitive_id"]))
    assert diff.mean() < 1e-3
    return hit.mean(), diff.sum()


def test_primary_hits_cornell(gpu_ctx, cornell):
    sc, sid, osc, cam = cornell
    frac, ties = _primary_checks(gpu_ctx, sid, osc, cam, 256, 256)
    assert frac > 0.9


def test_primary_hits_soup(gpu_ctx, soup_small):
    sc, sid, osc, cam = soup_small
    _primary_checks(gpu_ctx, sid, osc, cam, 320, 180)


def _random_rays(n, seed):
    from merian_gb300 import _native as N
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, N.RAY_DTYPE)
    rays["origin"] = rng.uniform(-0.1, 1.1, size=(n, 3))
    d = rng.normal(size=(n, 3))
    rays["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"] = 0.0
    rays["tmax"] = np.where(rng.uniform(size=n) < 0.2, rng.uniform(0.01, 0.5, size=n), 1e7)
    return rays


@pytest.mark.parametrize("which", ["cornell", "soup_small"])
def test_incoherent_rays_match_oracle(gpu_ctx, which, request):
    import torch
    from merian_gb300 import _native as N
    sc, sid, osc, cam = request.getfixturevalue(which)
    rays = _random_rays(200_000, 11)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(rays) * N.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr())
    gpu_ctx.synchronize()
    g = d_hits.cpu().numpy().view(N.HIT_DTYPE)
    o, _, _ = osc.trace_rays(rays, fp64=False, hit_dtype=N.HIT_DTYPE)
    assert np.array_equal(g["geometry_index"], o["geometry_index"])
    assert np.array_equal(g["primitive_id"], o["primitive_id"])
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
    # occlusion queries agree with the existence of a closest hit
    gpu_ctx.trace(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr(), any_hit=True)
    gpu_ctx.synchronize()
    ga = d_hits.cpu().numpy().view(N.HIT_DTYPE)
    assert np.array_equal(ga["geometry_index"] != 0xFFFFFFFF, o["geometry_index"] != 0xFFFFFFFF)


def _z_rmse(samples, gm, gv, gn):
    """z scores, relative RMSE and the RMSE sampling noise alone explains, of the per-frame GPU
    estimates `samples` (frames x pixels [x channels]) against the fixture's mean gm, per-sample
    variance gv over gn samples."""
    frames = samples.shape[0]
    m = samples.mean(0)
    se_g = samples.std(0, ddof=1) / np.sqrt(frames)
    se_o = np.sqrt(gv / gn)
    # FP32 floor: a zero-variance pixel (the environment seen directly) still differs from the
    # FP64 value by float round-off of the radiance itself
    se_fp32 = 1e-5 * np.abs(gm)
    se = np.sqrt(se_g ** 2 + se_o ** 2 + se_fp32 ** 2)
    ok = se > 0
    z = (m - gm)[ok] / se[ok]
    scale = max(np.mean(gm), 1e-12)
    rel_rmse = np.sqrt(np.mean((m - gm) ** 2)) / scale
    # RMSE an unbiased pair of estimators shows from sampling noise alone
    noise_rmse = np.sqrt(np.mean(se ** 2)) / scale
    return z, rel_rmse, noise_rmse


def _stat_compare(gpu_ctx, sid, cam, g, nee, rr, frames=8, spp=4096, lum2=False):
    """GPU per-pixel means (frames x spp samples; the standard error from the spread across
    frames, 16 frames so that it is itself well estimated) vs the FP64 fixture;
    with lum2 also the `a` channel against the fixture's mean squared luminance."""
    from merian_gb300 import scene as S
    pixels = g["pixels"]
    w, h, L = int(g["width"]), int(g["height"]), int(g["max_path_length"])
    outs = []
    for f in range(frames):
        params, keep = S.render_params(w, h, spp, L, pixels=pixels, nee=nee, rr_depth=rr,
                                       frame=1000 + f)
        outs.append(gpu_ctx.render(sid, cam, params).astype(np.float64))
    outs = np.stack(outs)
    gn = int(g["spp"])
    rgb = _z_rmse(outs[:, :, :3], g["mean"], g["var"], gn)
    if not lum2:
        return rgb
    return rgb, _z_rmse(outs[:, :, 3], g["lum2"], g["var_lum2"], gn)


def _assert_converged(z, rel_rmse, noise_rmse):
    # bias check: the RMSE is explained by the two estimators' sampling noise
    assert np.mean(np.abs(z) > 3) < 0.02
    assert np.mean(z ** 2) < 1.5
    assert rel_rmse < 1.25 * noise_rmse + 1e-4


def _check_estimator(gpu_ctx, which, sid, cam, nee, rr, frames, spp):
    g = golden(which)
    bsdf_only = not nee and rr == 0
    res = _stat_compare(gpu_ctx, sid, cam, g, nee, rr, frames=frames, spp=spp, lum2=bsdf_only)
    rgb, a = (res if bsdf_only else (res, None))
    z, rel_rmse, noise = rgb
    print(f"{which} nee={nee} rr={rr}: rel RMSE {rel_rmse:.4%} (noise {noise:.4%}), "
          f"max|z| {np.abs(z).max():.2f}")
    _assert_converged(z, rel_rmse, noise)
    if a is not None:
        za, rel_a, noise_a = a
        print(f"{which} a channel (mean luminance^2): rel RMSE {rel_a:.4%} "
              f"(noise {noise_a:.4%}), max|z| {np.abs(za).max():.2f}")
        _assert_converged(za, rel_a, noise_a)


@pytest.mark.parametrize("nee,rr", [(False, 0), (True, 0), (True, 3)],
                         ids=["bsdf", "nee", "nee_rr"])
def test_render_cornell_converges_to_oracle(gpu_ctx, cornell, nee, rr):
    sc, sid, osc, cam = cornell
    _check_estimator(gpu_ctx, "cornell", sid, cam, nee, rr, frames=16, spp=2048)


@pytest.mark.parametrize("nee,rr", [(False, 0), (True, 3)], ids=["bsdf", "nee_rr"])
def test_render_soup_converges_to_oracle(gpu_ctx, soup_small, nee, rr):
    sc, sid, osc, cam = soup_small
    _check_estimator(gpu_ctx, "soup_small", sid, cam, nee, rr, frames=16, spp=1024)


@pytest.mark.parametrize("nee,rr", [(False, 0), (True, 3)], ids=["bsdf", "nee_rr"])
def test_render_headline_soup_converges_to_oracle(gpu_ctx, soup_1m, nee, rr):
    """The benchmarked configuration (1M triangles, 2048x1024 environment, 1080p camera, path
    length 8) against its 65,536-spp FP64 fixture."""
    sc, sid, osc, cam = soup_1m
    _check_estimator(gpu_ctx, "soup_1m", sid, cam, nee, rr, frames=16, spp=4096)


def test_headline_estimator_within_one_percent(gpu_ctx, soup_1m):
    """The benchmarked estimator (NEE + roulette from path length 3) converges to the reference's
    BSDF-only estimator: on the 64 pixels of the deep FP64 fixture (2^22 spp, its own noise a
    third of a percent) the GPU at 2^22 spp per pixel lands within 1 % relative RMSE, and every
    pixel within 4 combined standard errors."""
    from merian_gb300 import scene as S
    sc, sid, osc, cam = soup_1m
    g = golden("soup_1m_deep")
    n = int(g["spp"])
    halves = []
    for f in range(2):  # two independent halves: their spread is the GPU estimate's noise
        p, keep = S.render_params(int(g["width"]), int(g["height"]), n // 2,
                                  int(g["max_path_length"]), pixels=g["pixels"], nee=True,
                                  rr_depth=3, frame=2000 + f)
        halves.append(gpu_ctx.render(sid, cam, p)[:, :3].astype(np.float64))
    m = 0.5 * (halves[0] + halves[1])
    scale = float(np.mean(g["mean"]))
    rel_rmse = np.sqrt(np.mean((m - g["mean"]) ** 2)) / scale
    se_o = np.sqrt(g["var"] / n)
    # the GPU estimate's standard error: the spread of its two halves, at least the oracle's
    se_g = np.maximum(se_o, 0.5 * np.abs(halves[0] - halves[1]))
    se = np.sqrt(se_o ** 2 + se_g ** 2 + (1e-5 * np.abs(g["mean"])) ** 2)
    z = (m - g["mean"]) / np.maximum(se, 1e-12)
    print(f"soup_1m deep: rel RMSE {rel_rmse:.4%}, oracle noise "
          f"{np.sqrt(np.mean(se_o ** 2)) / scale:.4%}, max|z| {np.abs(z).max():.2f}")
    assert rel_rmse < 0.01
    assert np.abs(z).max() < 4.5


def test_render_deterministic_and_subset_consistent(gpu_ctx, cornell):
    from merian_gb300 import scene as S
    sc, sid, osc, cam = cornell
    p, _ = S.render_params(256, 256, 16, 5, frame=3)
    a = gpu_ctx.render(sid, cam, p)
    b = gpu_ctx.render(sid, cam, p)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    pix = np.arange(0, 65536, 97, dtype=np.uint32)
    ps, keep = S.render_params(256, 256, 16, 5, frame=3, pixels=pix)
    c = gpu_ctx.render(sid, cam, ps)
    assert np.array_equal(c.view(np.uint32), a[pix].view(np.uint32))


def test_triangle_records_and_index_path_agree(gpu_ctx, cornell):
    """Shading reads a triangle's vertices from its 80-byte record when every triangle has one
    first vertex, and through the index buffer when two geometries over one triangle range
    disagree on it. The Cornell box plus a geometry that is never hit (instance mask 0) over the
    range of a diffuse one with its first vertex moved by one takes the index path and renders the
    same bits."""
    import dataclasses
    from merian_gb300 import scene as S
    sc, sid, osc, cam = cornell
    geo = sc.geometries
    mats = sc.materials
    # a diffuse, non-emissive geometry whose indices stay in range when moved by one vertex
    g0 = next(g for g in range(len(geo))
              if mats[geo[g]["material_id"]]["model"] == 0
              and not np.any(mats[geo[g]["material_id"]]["emission"])
              and (geo[g]["first_vertex"] + sc.indices[geo[g]["first_triangle"]:
                   geo[g]["first_triangle"] + geo[g]["triangle_count"]].max() + 1)
              < len(sc.vertices))
    extra = geo[g0:g0 + 1].copy()
    extra["first_vertex"] += 1
    extra["instance_mask"] = 0
    sc2 = dataclasses.replace(sc, geometries=np.concatenate([geo, extra]))
    sid2 = gpu_ctx.upload(sc2)
    try:
        b1, b2 = gpu_ctx.scene_stats(sid)["bytes"], gpu_ctx.scene_stats(sid2)["bytes"]
        # the first scene holds the records (80 B per triangle), the second does not (its tree
        # is larger by the extra geometry's 128 triangles, far less than the records)
        assert b1 - b2 > 40 * sc.triangle_count, (b1, b2)
        p, _ = S.render_params(256, 256, 8, 6, nee=True, rr_depth=3, frame=11)
        a = gpu_ctx.render(sid, cam, p)
        b = gpu_ctx.render(sid2, cam, p)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    finally:
        gpu_ctx.destroy_scene(sid2)


def test_render_first_bounce_tracks_fp32_oracle(gpu_ctx, cornell):
    """Same RNG stream and same primary hit: with one bounce (path length 2) the GPU and the FP32
    oracle agree per pixel to float round-off of the BSDF sampling."""
    from merian_gb300 import scene as S
    sc, sid, osc, cam = cornell
    pix = np.arange(0, 65536, 61, dtype=np.uint32)
    p, keep = S.render_params(256, 256, 4, 2, pixels=pix, frame=5)
    g = gpu_ctx.render(sid, cam, p).astype(np.float64)
    o, _, _ = osc.render(cam, p, fp64=False)
    close = np.isclose(g[:, :3], o[:, :3], rtol=1e-3, atol=1e-5).all(axis=1)
    assert close.mean() > 0.97, close.mean()


def test_render_stats_and_edge_cases(gpu_ctx, cornell):
    from merian_gb300 import scene as S
    from merian_gb300 import _native as N
    sc, sid, osc, cam = cornell
    p, _ = S.render_params(64, 48, 8, 5)
    out, st = gpu_ctx.render(sid, cam, p, stats=True)
    assert out.shape == (64 * 48, 4) and np.all(np.isfinite(out))
    assert st.samples == 64 * 48 * 8 and st.rays >= 64 * 48 and st.device_ms > 0
    # zero samples: output is cleared, no work
    p0, _ = S.render_params(8, 8, 0, 5)
    assert np.all(gpu_ctx.render(sid, cam, p0) == 0)
    # path length 1: emission on primary only
    p1, _ = S.render_params(256, 256, 2, 1)
    o1 = gpu_ctx.render(sid, cam, p1)
    assert set(np.unique(o1[:, 0])) <= {0.0, 15.0}
    # invalid arguments are rejected, not run
    with pytest.raises(N.GbptError):
        gpu_ctx.render(sid + 1000, cam, p)
    bad, _ = S.render_params(8, 8, 1, 0)
    with pytest.raises(N.GbptError):
        gpu_ctx.render(sid, cam, bad)

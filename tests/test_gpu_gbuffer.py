"""GPU: the GBuffer (Raytraced) node and RenderPT's "demodulate albedo".

GBuffer texels against the FP32 oracle restatement of gbuffer_rt.slang (same traversal result,
so the hit ids and half barycentrics are identical; the float fields agree to FP32 round-off:
linear_z 1e-6 relative, normals within 1e-4 rad, albedo and emission 2e-5 relative, grad_z to
half precision). Demodulation: every sample is divided by the GBuffer albedo floored at 1e-2, so
the demodulated mean times that albedo equals the plain mean to FP32 round-off (1e-5 relative),
and the demodulated estimate converges to the FP64 oracle's demodulated estimate (z-test as in
the render parity tests)."""
import numpy as np
import pytest

from oracle import binding as O

pytestmark = pytest.mark.gpu


def decode_normal(enc):
    enc = np.asarray(enc, np.uint32)
    x = (enc & 0xFFFF).astype(np.uint16).view(np.int16).astype(np.float64) / 32767.0
    y = (enc >> 16).astype(np.uint16).view(np.int16).astype(np.float64) / 32767.0
    x, y = np.clip(x, -1, 1), np.clip(y, -1, 1)
    z = 1.0 - np.abs(x) - np.abs(y)
    t = np.maximum(-z, 0.0)
    x = x + np.where(x >= 0, -t, t)
    y = y + np.where(y >= 0, -t, t)
    v = np.stack([x, y, z], -1)
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def half2(u):
    u = np.asarray(u, np.uint32)
    lo = (u & 0xFFFF).astype(np.uint16).view(np.float16).astype(np.float64)
    hi = (u >> 16).astype(np.uint16).view(np.float16).astype(np.float64)
    return lo, hi


def gbuffer_gpu(ctx, sid, cam, w, h):
    import torch
    from merian_gb300 import _native as N
    import ctypes as C
    buf = torch.zeros(w * h * 16, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    N.check(ctx.lib.gbpt_gbuffer(ctx.handle, sid, C.byref(cam), w, h, 0xFF, buf.data_ptr()))
    ctx.synchronize()
    return buf.cpu().numpy().view(N.GBUFFER_DTYPE)


@pytest.fixture(scope="module", params=["cornell", "soup"])
def scene(request, gpu_ctx):
    from merian_gb300 import scene as S
    if request.param == "cornell":
        sc = S.cornell()
        cam, w, h = S.workload_camera("cornell-256-16spp"), 256, 256
    else:
        sc = S.soup(S.BASE_SEED, 200_000, 256, (256, 128))
        w, h = 320, 180
        cam = S.look_at((0.5, 0.5, -1.2), (0.5, 0.5, 0.5), (0, 1, 0), 45.0, w / h)
    sid = gpu_ctx.upload(sc)
    yield request.param, sc, sid, O.OracleScene(sc), cam, w, h
    gpu_ctx.destroy_scene(sid)


def test_gbuffer_matches_oracle(gpu_ctx, scene):
    from merian_gb300 import _native as N
    name, sc, sid, osc, cam, w, h = scene
    g = gbuffer_gpu(gpu_ctx, sid, cam, w, h)
    o = osc.gbuffer(cam, w, h, texel_dtype=N.GBUFFER_DTYPE)
    for k in ("instance_id", "primitive_id", "geometry_index", "instance_index", "barycentrics"):
        assert np.array_equal(g[k], o[k]), k
    hit = g["instance_id"] == 0
    assert hit.mean() > (0.9 if name == "cornell" else 0.3)
    assert np.allclose(g["linear_z"], o["linear_z"], rtol=1e-6)
    assert np.all(g["linear_z"][~hit] == 65504.0)
    dots = np.sum(decode_normal(g["encoded_normal"]) * decode_normal(o["encoded_normal"]), -1)
    assert dots.min() > 1 - 1e-4
    assert np.allclose(g["albedo"], o["albedo"], rtol=2e-5, atol=1e-6)
    assert np.allclose(g["emission"], o["emission"], rtol=2e-5, atol=1e-6)
    assert np.all(g["motion"] == 0) and np.allclose(g["delta_z"], 0, atol=1e-5)
    gl, gh = half2(g["grad_z"][hit])
    ol, oh = half2(o["grad_z"][hit])
    fin = np.isfinite(gl) & np.isfinite(ol) & (np.abs(ol) < 1e3)
    assert np.allclose(gl[fin], ol[fin], rtol=2e-3, atol=2e-3)
    fin = np.isfinite(gh) & np.isfinite(oh) & (np.abs(oh) < 1e3)
    assert np.allclose(gh[fin], oh[fin], rtol=2e-3, atol=2e-3)
    if name == "cornell":  # diffuse materials: the albedo is the base colour
        mats = sc.materials[sc.geometries["material_id"][g["geometry_index"][hit]]]
        diff = mats["model"] == 0
        assert np.array_equal(g["albedo"][hit][diff], mats["base_color"][diff])


def test_demodulation_divides_by_gbuffer_albedo(gpu_ctx, scene):
    from merian_gb300 import scene as S
    name, sc, sid, osc, cam, w, h = scene
    g = gbuffer_gpu(gpu_ctx, sid, cam, w, h)
    a = np.maximum(g["albedo"].astype(np.float64), 1e-2)
    kw = dict(nee=True, rr_depth=3, frame=9) if name == "soup" else dict(frame=9)
    L = 8 if name == "soup" else 5
    p, _ = S.render_params(w, h, 8, L, **kw)
    plain = gpu_ctx.render(sid, cam, p).astype(np.float64)
    p.demodulate_albedo = 1
    demod = gpu_ctx.render(sid, cam, p).astype(np.float64)
    assert np.allclose(demod[:, :3] * a, plain[:, :3], rtol=1e-5, atol=1e-7)


def test_demodulated_estimate_converges_to_oracle(gpu_ctx, scene):
    from merian_gb300 import scene as S
    name, sc, sid, osc, cam, w, h = scene
    rng = np.random.default_rng(11)
    pix = np.sort(rng.choice(w * h, 48, replace=False)).astype(np.uint32)
    kw = dict(nee=True, rr_depth=3) if name == "soup" else {}
    L = 8 if name == "soup" else 5
    spp = 4096
    p, keep = S.render_params(w, h, spp, L, pixels=pix, frame=3, **kw)
    p.demodulate_albedo = 1
    gm = gpu_ctx.render(sid, cam, p)[:, :3].astype(np.float64)
    p2, keep2 = S.render_params(w, h, spp, L, pixels=pix, frame=77, **kw)
    p2.demodulate_albedo = 1
    om, osq, _ = osc.render(cam, p2, fp64=True)
    om = om[:, :3]
    var = np.maximum(osq - om * om, 0.0)
    se = np.sqrt(2 * var / spp) + 1e-5 * np.abs(om) + 1e-7
    z = (gm - om) / se
    assert np.mean(np.abs(z) > 3) <= 0.03 and np.mean(z * z) < 1.6

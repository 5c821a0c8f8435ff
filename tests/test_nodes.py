"""The graph nodes either side of the renderer: PFM files (CPU), graph JSON loading and RenderPT
properties (CPU), Accumulate and the error metrics on the GPU against numpy, and a
render -> accumulate -> image write graph against individually rendered frames."""
import math

import numpy as np
import pytest

from conftest import ROOT


def test_pfm_round_trip(native, tmp_path):
    from merian_gb300 import node
    rng = np.random.default_rng(1)
    img = rng.normal(size=(7, 5, 4)).astype(np.float32)
    p = tmp_path / "a.pfm"
    node.write_pfm(str(p), img, 5, 7)
    raw = p.read_bytes()
    assert raw.startswith(b"PF\n5 7\n-1\n")
    body = np.frombuffer(raw[len(b"PF\n5 7\n-1\n"):], np.float32).reshape(7, 5, 3)
    assert np.array_equal(body, img[::-1, :, :3])  # bottom row first, alpha dropped
    back = node.read_pfm(str(p), 4)
    assert np.array_equal(back[..., :3], img[..., :3]) and np.all(back[..., 3] == 1)
    grey = img[..., :1].copy()
    q = tmp_path / "g.pfm"
    node.write_pfm(str(q), grey, 5, 7)
    assert q.read_bytes().startswith(b"Pf\n")
    assert np.array_equal(node.read_pfm(str(q), 1), grey)
    assert np.array_equal(node.read_pfm(str(q), 3)[..., 2], grey[..., 0])


def test_pfm_big_endian_and_errors(native, tmp_path):
    from merian_gb300 import node
    img = np.arange(12, dtype=np.float32).reshape(2, 2, 3)
    p = tmp_path / "be.pfm"
    p.write_bytes(b"PF\n2 2\n1.0\n" + img[::-1].astype(">f4").tobytes())
    assert np.array_equal(node.read_pfm(str(p), 3), img)
    bad = tmp_path / "bad.pfm"
    bad.write_bytes(b"P6\n2 2\n255\n")
    with pytest.raises(Exception):
        node.read_pfm(str(bad), 3)


PT_JSON = {
    "nodes": {
        "render": {"type": "Render (Path-traced)", "enabled": True,
                   "outputs": ["irradiance->accumulate.src"],
                   "properties": {"0": True, "1": True, "2": True, "3": True, "4": True,
                                  "5": True, "6": True, "7": True, "emission on primary": True,
                                  "max path length": 5, "samples per pixel": 2}},
        "accumulate": {"type": "Accumulate", "outputs": ["out->write.src"],
                       "properties": {"alpha": 1.0, "inf history": True}},
        "write": {"type": "Image Write", "properties": {"filename": "frame_{iteration}.pfm",
                                                        "enable": False}},
    }
}


def test_graph_json_and_properties(native):
    from merian_gb300 import node
    g = node.Graph(None, PT_JSON)
    assert g.order == ["render", "accumulate", "write"]
    r = g.nodes["render"]
    assert r.props["samples per pixel"] == 2 and r.instance_mask() == 0xFF
    assert r.properties({"1": False}) == 0 and r.instance_mask() == 0xFD
    with pytest.raises(ValueError):
        r.properties({"no such key": 1})
    with pytest.raises(ValueError):
        r.properties({"irradiance format": "R8G8B8A8Unorm"})
    assert node.RenderPT.DEFAULTS["samples per pixel"] == 1
    assert node.RenderPT.DEFAULTS["max path length"] == 5
    bad = {"nodes": {"x": {"type": "Bloom"}}}
    with pytest.raises(ValueError):
        node.Graph(None, bad)


@pytest.mark.gpu
def test_accumulate_running_mean(gpu_ctx):
    import torch
    from merian_gb300 import _native as N
    rng = np.random.default_rng(3)
    frames = rng.uniform(0, 2, size=(6, 1000, 4)).astype(np.float32)
    out = torch.zeros((1000, 4), device="cuda")
    hist = torch.zeros(1000, device="cuda")
    torch.cuda.synchronize()
    for i, f in enumerate(frames):
        src = torch.from_numpy(f).cuda()
        torch.cuda.synchronize()
        N.check(gpu_ctx.lib.gbpt_accumulate(gpu_ctx.handle, src.data_ptr(), out.data_ptr(),
                                            hist.data_ptr(), 1000, 1.0, math.inf, int(i == 0)))
        gpu_ctx.synchronize()
    mean = frames.astype(np.float64).mean(axis=0)
    assert np.allclose(out.cpu().numpy(), mean, rtol=1e-5, atol=1e-6)
    assert np.all(hist.cpu().numpy() == 6)
    # the reference's update, restated in float32 with the same rounding order
    ref = frames[0].copy()
    for n, f in enumerate(frames[1:], start=2):
        a = np.float32(max(0.0, np.float32(1) / np.float32(n)))
        ref = (ref + a * (f - ref)).astype(np.float32)
    assert np.array_equal(out.cpu().numpy(), ref)
    # alpha = 0 (merian's default) keeps only the newest frame (lerp with weight 1: one
    # rounding of prev + (src - prev))
    N.check(gpu_ctx.lib.gbpt_accumulate(gpu_ctx.handle, src.data_ptr(), out.data_ptr(),
                                        hist.data_ptr(), 1000, 0.0, math.inf, 0))
    gpu_ctx.synchronize()
    assert np.allclose(out.cpu().numpy(), frames[-1], rtol=1e-6, atol=1e-7)


@pytest.mark.gpu
def test_error_metrics(gpu_ctx):
    import torch
    from merian_gb300 import _native as N
    import ctypes as C
    rng = np.random.default_rng(4)
    a = rng.normal(size=(5000, 4)).astype(np.float32)
    b = rng.normal(size=(5000, 4)).astype(np.float32)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    torch.cuda.synchronize()
    out = (C.c_double * 8)()
    N.check(gpu_ctx.lib.gbpt_error_metrics(gpu_ctx.handle, ta.data_ptr(), tb.data_ptr(), 5000, out))
    d = a.astype(np.float64) - b.astype(np.float64)
    assert np.allclose(list(out)[:4], (d * d).mean(axis=0), rtol=1e-12)
    assert np.allclose(list(out)[4:], np.abs(d).mean(axis=0), rtol=1e-12)


@pytest.mark.gpu
def test_graph_render_accumulate_write(gpu_ctx, tmp_path):
    import torch
    from merian_gb300 import node
    from merian_gb300 import scene as S
    sid = gpu_ctx.upload(S.cornell())
    cam = S.workload_camera("cornell-256-16spp")
    cfg = {"nodes": dict(PT_JSON["nodes"])}
    cfg["nodes"]["write"] = {"type": "Image Write",
                             "properties": {"filename": str(tmp_path / "f_{iteration}.pfm"),
                                            "every": 4}}
    g = node.Graph(gpu_ctx, cfg)
    outs = g.run(sid, cam, (64, 64), iterations=4)
    acc = outs["accumulate.out"].cpu().numpy().reshape(-1, 4)
    # the same four frames rendered one by one (frame = iteration)
    frames = []
    for it in range(4):
        p, _ = S.render_params(64, 64, 2, 5, frame=it)
        frames.append(gpu_ctx.render(sid, cam, p))
    mean = np.mean(np.stack(frames).astype(np.float64), axis=0)
    assert np.allclose(acc, mean, rtol=1e-5, atol=1e-6)
    written = g.nodes["write"].written
    assert written == [str(tmp_path / "f_0.pfm")]
    gpu_ctx.destroy_scene(sid)

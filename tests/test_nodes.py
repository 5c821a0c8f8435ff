"""The graph nodes either side of the renderer: PFM files (CPU), graph JSON loading and RenderPT
properties (CPU), Accumulate and the error metrics on the GPU against numpy, and a
render -> accumulate -> image write graph against individually rendered frames."""
import ctypes as C
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
        "write": {"type": "Image Write",
                  "properties": {"format": "PFM", "filename": "frame_{record_iteration}"}},
    }
}


def test_graph_json_and_properties(native):
    """The C++ node graph checked without a context: run order, merian's property keys and
    defaults, NodeStatusFlags, and the errors and warnings of bad graphs and values."""
    from merian_gb300 import _native as N
    from merian_gb300 import node
    g = node.Graph(None, PT_JSON)
    assert g.order == ["render", "accumulate", "write"]
    assert g.node_type("render") == "Render (Path-traced)" and g.warnings == []
    p = g.properties("render")
    assert p["samples per pixel"] == 2 and p["max path length"] == 5 and p["seed"] == 0
    assert p["shader execution reordering"] is False and p["irradiance format"] == "R32G32B32A32Sfloat"
    assert g.set_property("render", "1", False) == 0 and g.properties("render", "1") is False
    for key, value in [("no such key", 1), ("irradiance format", "R8G8B8A8Unorm"),
                       ("samples per pixel", "x"), ("samples per pixel", 1.5),
                       ("max path length", 0), ("emission on primary", 1)]:
        with pytest.raises(N.GbptError):
            g.set_property("render", key, value)
    assert g.properties("render", "samples per pixel") == 2  # a refused value changes nothing
    # merian's defaults (render_pt.hpp, accumulate.hpp, image_write.hpp)
    d = node.Graph(None, {"nodes": {"r": {"type": "Render (Path-traced)"},
                                    "a": {"type": "Accumulate"}, "w": {"type": "Image Write"}}})
    r = d.properties("r")
    assert (r["samples per pixel"], r["max path length"], r["emission on primary"]) == (1, 5, True)
    assert all(r[str(b)] for b in range(8))
    a = d.properties("a")
    assert a["alpha"] == 0.0 and a["max history"] is None  # infinity
    w = d.properties("w")
    assert w["format"] == "PNG" and w["filename"] == "image_{image_index_total:04}"
    assert w["iteration"] == 1 and w["advanced"]["stop at run"] == -1
    # buttons act once; "inf history" sets the history limit to infinity
    assert d.set_property("a", "max history", 16) == 0 and d.properties("a", "max history") == 16
    d.set_property("a", "inf history", True)
    assert d.properties("a", "max history") is None and d.properties("a", "inf history") is False
    # values this library cannot honour are refused, as merian's node_error
    for node_name, key, value in [("a", "firefly filter enable", True), ("a", "hard clamp", 10),
                                  ("a", "adaptivity", 0.5), ("w", "format", "PNG"),
                                  ("w", "trigger", "frametime"), ("w", "advanced/scale", 0.5)]:
        with pytest.raises(N.GbptError):
            d.set_property(node_name, key, value)
    assert d.set_property("w", "advanced/stop at run", 7) == 0
    assert d.properties("w")["advanced"]["stop at run"] == 7
    # NEEDS_RECONNECT when a connector layout changes
    gb = node.Graph(None, {"nodes": {"g": {"type": "GBuffer (Raytraced)"}}})
    assert gb.properties("g", "width") == 1920 and gb.properties("g", "height") == 1080
    assert gb.set_property("g", "width", 640) == node.NEEDS_RECONNECT
    assert gb.set_property("g", "width", 640) == 0
    # unknown keys in a graph JSON are ignored with a warning; bad graphs are refused
    u = node.Graph(None, {"nodes": {"r": {"type": "Render (Path-traced)",
                                          "properties": {"no such key": 1}}}})
    assert len(u.warnings) == 1 and "no such key" in u.warnings[0]
    off = node.Graph(None, {"nodes": {"r": {"type": "Render (Path-traced)",
                                            "outputs": ["irradiance->x.src"]},
                                      "x": {"type": "Bloom", "enabled": False}}})
    assert off.order == ["r"] and len(off.warnings) == 1
    bad = [{"nodes": {"x": {"type": "Bloom"}}},
           {"nodes": {"r": {"type": "Render (Path-traced)", "outputs": ["nope->a.src"]},
                      "a": {"type": "Accumulate"}}},
           {"nodes": {"r": {"type": "Render (Path-traced)", "outputs": ["irradiance->a.nope"]},
                      "a": {"type": "Accumulate"}}},
           {"nodes": {"a": {"type": "Accumulate", "outputs": ["out->b.src"]},
                      "b": {"type": "Accumulate", "outputs": ["out->a.src"]}}},
           {"nodes": {"r": {"type": "Render (Path-traced)", "properties": {"seed": -1}}}},
           {"no nodes": {}}]
    for cfg in bad:
        with pytest.raises(N.GbptError):
            node.Graph(None, cfg)
    with pytest.raises(N.GbptError):
        node.Graph(None, "{\"nodes\": {}} trailing")
    with pytest.raises(N.GbptError):  # a graph without a context does not run
        from merian_gb300 import scene as S
        g.run(0, S.look_at((0, 0, 0), (0, 0, 1), (0, 1, 0), 40.0, 1.0), (8, 8))


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
    """pt.json's render -> accumulate -> Image Write: the accumulated image is the mean of the
    frames rendered one by one (RNG lane 3 = the graph iteration), and Image Write captures at
    its 1-indexed iterations 2, then 2 * 2 + 0 = 4 ("iteration power" 2, "iteration offset" 0)."""
    from merian_gb300 import node
    from merian_gb300 import scene as S
    sid = gpu_ctx.upload(S.cornell())
    cam = S.workload_camera("cornell-256-16spp")
    cfg = {"nodes": dict(PT_JSON["nodes"])}
    cfg["nodes"]["write"] = {"type": "Image Write",
                             "properties": {"format": "PFM", "enable": True,
                                            "filename": str(tmp_path / "f_{record_iteration}"),
                                            "iteration": 2, "iteration power": 2,
                                            "iteration offset": 0}}
    try:
        with node.Graph(gpu_ctx, cfg) as g:
            g.run(sid, cam, (64, 64), iterations=4)
            acc = g.output("accumulate.out")
            assert acc.shape == (64, 64, 4)
            assert g.output("accumulate.history").shape == (64, 64, 1)
            assert np.all(g.output("accumulate.history") == 4)
            assert g.properties("write", "iteration") == 8 and g.properties("write", "enable")
        frames = []
        for it in range(4):
            p, _ = S.render_params(64, 64, 2, 5, frame=it)
            frames.append(gpu_ctx.render(sid, cam, p))
        mean = np.mean(np.stack(frames).astype(np.float64), axis=0)
        assert np.allclose(acc.reshape(-1, 4), mean, rtol=1e-5, atol=1e-6)
        assert sorted(x.name for x in tmp_path.iterdir()) == ["f_2.pfm", "f_4.pfm"]
        f4 = node.read_pfm(str(tmp_path / "f_4.pfm"), 4)
        assert np.array_equal(f4[..., :3], acc[..., :3])
        f2 = node.read_pfm(str(tmp_path / "f_2.pfm"), 4)
        assert np.allclose(f2[..., :3].reshape(-1, 3), np.mean(np.stack(frames[:2]), 0)[:, :3],
                           rtol=1e-5, atol=1e-6)
    finally:
        gpu_ctx.destroy_scene(sid)


@pytest.mark.gpu
def test_graph_gbuffer_and_error_plot(gpu_ctx):
    """A GBuffer (Raytraced) node gives the renderer its extent; its texels equal gbpt_gbuffer's.
    Error Plot's MSE / RMSE / MAE of two renders (seeds 0 and 1000) match numpy, with a history
    of one value per iteration."""
    import torch
    from merian_gb300 import _native as N
    from merian_gb300 import node
    from merian_gb300 import scene as S
    sid = gpu_ctx.upload(S.cornell())
    cam = S.workload_camera("cornell-256-16spp")
    cfg = {"nodes": {
        "gbuffer": {"type": "GBuffer (Raytraced)", "properties": {"width": 48, "height": 32},
                    "outputs": ["gbuffer->a.gbuffer", "gbuffer->b.gbuffer"]},
        "a": {"type": "Render (Path-traced)", "outputs": ["irradiance->plot.reference"],
              "properties": {"samples per pixel": 4}},
        "b": {"type": "Render (Path-traced)", "outputs": ["irradiance->plot.input"],
              "properties": {"samples per pixel": 4, "seed": 1000}},
        "plot": {"type": "Error Plot", "properties": {"Metric": "MSE", "History": 2}}}}
    try:
        with node.Graph(gpu_ctx, cfg) as g:
            assert g.order == ["gbuffer", "a", "b", "plot"]
            g.run(sid, cam, (64, 64), iterations=3)
            ra, rb = g.output("a.irradiance"), g.output("b.irradiance")
            assert ra.shape == (32, 48, 4)
            p, _ = S.render_params(48, 32, 4, 5, frame=2)
            assert np.array_equal(ra.reshape(-1, 4), gpu_ctx.render(sid, cam, p))
            p, _ = S.render_params(48, 32, 4, 5, frame=1002)
            assert np.array_equal(rb.reshape(-1, 4), gpu_ctx.render(sid, cam, p))
            gb = g.output("gbuffer.gbuffer")
            assert gb.shape == (32, 48, 16)
            ref = torch.zeros(48 * 32 * 64, dtype=torch.uint8, device="cuda")
            N.check(gpu_ctx.lib.gbpt_gbuffer(gpu_ctx.handle, sid, C.byref(cam), 48, 32, 0xFF,
                                             ref.data_ptr()))
            gpu_ctx.synchronize()
            assert np.array_equal(gb.reshape(-1).view(np.uint8), ref.cpu().numpy())
            texels = ref.cpu().numpy().view(N.GBUFFER_DTYPE)
            em = g.output("gbuffer.emission").reshape(-1, 4)
            assert np.array_equal(em[:, :3], texels["emission"]) and np.all(em[:, 3] == 1)
            d = ra.astype(np.float64) - rb.astype(np.float64)
            mse = (d * d).reshape(-1, 4).mean(axis=0)
            assert np.allclose(g.output("plot.error").reshape(4), mse, rtol=1e-6)
            assert g.output("plot.history").shape == (1, 2, 4)
            g.set_property("plot", "Metric", "MAE")
            g.run(sid, cam, (64, 64), iterations=1)
            ra, rb = g.output("a.irradiance"), g.output("b.irradiance")
            mae = np.abs(ra.astype(np.float64) - rb).reshape(-1, 4).mean(axis=0)
            assert np.allclose(g.output("plot.error").reshape(4), mae, rtol=1e-6)
    finally:
        gpu_ctx.destroy_scene(sid)


@pytest.mark.gpu
def test_graph_scene_file_node(gpu_ctx, tmp_path):
    """A "GLTF Scene" node loads its file when the graph first runs and hands the scene and the
    file's camera to the renderer: the image equals loading the file and rendering it directly."""
    from test_gltf import build_scene
    from merian_gb300 import _native as N
    from merian_gb300 import node
    from merian_gb300 import scene as S
    path, _ = build_scene(tmp_path, "glb")
    cfg = {"nodes": {"scene": {"type": "GLTF Scene", "properties": {"file": str(path)},
                               "outputs": ["scene->render.scene"]},
                     "render": {"type": "Render (Path-traced)",
                                "properties": {"samples per pixel": 2}}}}
    with node.Graph(gpu_ctx, cfg) as g:
        g.run(0, None, (72, 48), iterations=2)
        img = g.output("render.irradiance")
    sc, cam, _, _ = S.load_gltf(path)
    sid = gpu_ctx.upload(sc)
    try:
        p, _ = S.render_params(72, 48, 2, 5, frame=1)
        assert np.array_equal(img.reshape(-1, 4), gpu_ctx.render(sid, cam, p))
    finally:
        gpu_ctx.destroy_scene(sid)
    cfg["nodes"]["scene"]["properties"]["file"] = str(tmp_path / "missing.glb")
    with node.Graph(gpu_ctx, cfg) as g:
        with pytest.raises(N.GbptError):
            g.run(0, None, (72, 48))


def test_graph_checkpoint_properties(native, tmp_path):
    """A checkpoint of a graph without a context carries the iteration count and every property
    (infinity as null) into a graph made from the same JSON."""
    from merian_gb300 import _native as N
    from merian_gb300 import node
    g = node.Graph(None, PT_JSON)
    g.set_property("render", "samples per pixel", 7)
    g.set_property("accumulate", "max history", 32)
    g.set_property("write", "advanced/stop at run", 9)
    g.save(tmp_path / "ck")
    state = (tmp_path / "ck" / "graph_state.json").read_text()
    assert '"iteration":0' in state
    h = node.Graph(None, PT_JSON)
    h.load(tmp_path / "ck")
    for name in ("render", "accumulate", "write"):
        assert h.properties(name) == g.properties(name)
    other = node.Graph(None, {"nodes": {"render": {"type": "Accumulate"}}})
    with pytest.raises(N.GbptError):
        other.load(tmp_path / "ck")
    with pytest.raises(N.GbptError):
        h.load(tmp_path / "missing")


@pytest.mark.gpu
def test_graph_checkpoint_resume(gpu_ctx, tmp_path):
    """Render -> Accumulate for 6 iterations equals 3 iterations, a checkpoint, a new graph
    loading it, and 3 more iterations, bit for bit (frame seeds continue from the iteration
    count; the accumulator and its history are restored exactly)."""
    from merian_gb300 import node
    from merian_gb300 import scene as S
    sid = gpu_ctx.upload(S.cornell())
    cam = S.workload_camera("cornell-256-16spp")
    cfg = {"nodes": {
        "render": {"type": "Render (Path-traced)", "outputs": ["irradiance->accumulate.src"],
                   "properties": {"samples per pixel": 1, "seed": 5}},
        "accumulate": {"type": "Accumulate", "outputs": ["out->plot.input"],
                       "properties": {"alpha": 1.0, "inf history": True}},
        "gt": {"type": "Render (Path-traced)", "outputs": ["irradiance->plot.reference"],
               "properties": {"samples per pixel": 4}},
        "plot": {"type": "Error Plot", "properties": {"Metric": "RMSE"}}}}
    try:
        with node.Graph(gpu_ctx, cfg) as g:
            g.run(sid, cam, (40, 24), iterations=6)
            full = g.output("accumulate.out")
            full_hist = g.output("plot.history")
        with node.Graph(gpu_ctx, cfg) as g:
            g.run(sid, cam, (40, 24), iterations=3)
            g.save(tmp_path / "ck")
        with node.Graph(gpu_ctx, cfg) as g:
            g.load(tmp_path / "ck")
            g.run(sid, cam, (40, 24), iterations=3)
            resumed = g.output("accumulate.out")
            assert np.all(g.output("accumulate.history") == 6)
            assert np.array_equal(g.output("plot.history"), full_hist)
        assert np.array_equal(resumed.view(np.uint32), full.view(np.uint32))
    finally:
        gpu_ctx.destroy_scene(sid)


def test_graph_cli_options(native):
    """pt.json's "cli" section: options name JSON pointers to node properties (RFC 6901
    escapes); setting one sets the property; pointers to nothing are dropped with a warning."""
    from merian_gb300 import _native as N
    from merian_gb300 import node
    cfg = dict(PT_JSON)
    cfg["cli"] = {"max-path-length": {"pointer": "/nodes/render/properties/max path length"},
                  "spp": {"pointer": "/nodes/render/properties/samples per pixel"},
                  "stop": {"pointer": "/nodes/write/properties/advanced/stop at run"},
                  "bad": {"pointer": "/nodes/nope/properties/x"}}
    g = node.Graph(None, cfg)
    assert set(g.options) == {"max-path-length", "spp", "stop"}
    assert len(g.warnings) == 1 and "bad" in g.warnings[0]
    g.set_option("spp", 16)
    g.set_option("max-path-length", 9)
    g.set_option("stop", 3)
    assert g.properties("render", "samples per pixel") == 16
    assert g.properties("render", "max path length") == 9
    assert g.properties("write")["advanced"]["stop at run"] == 3
    with pytest.raises(N.GbptError):
        g.set_option("nope", 1)
    with pytest.raises(N.GbptError):
        g.set_option("spp", "many")


def test_graph_json_round_trip(native):
    """Load -> store -> load gives the same graph (as merian's graph_load_store tests check):
    the stored JSON holds every property with its value, the edges and the cli options."""
    from merian_gb300 import node
    cfg = dict(PT_JSON)
    cfg["cli"] = {"spp": {"pointer": "/nodes/render/properties/samples per pixel"}}
    g = node.Graph(None, cfg)
    g.set_property("render", "seed", 11)
    stored = g.to_json()
    assert stored["cli"] == cfg["cli"]
    assert stored["nodes"]["render"]["outputs"] == ["irradiance->accumulate.src"]
    assert stored["nodes"]["render"]["properties"]["seed"] == 11
    assert stored["nodes"]["write"]["type"] == "Image Write"
    h = node.Graph(None, stored)
    assert h.to_json() == stored and h.order == g.order and h.warnings == []

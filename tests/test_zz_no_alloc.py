"""GPU test of gbpt_render_device_noalloc, the render entry point for callers that cannot allocate
device memory while they render (a host whose allocator owns the GPU, a real-time loop that must
not block in cudaMalloc/cudaFree, a fixed memory budget). It draws every scratch buffer from the
library's fixed device array, so its result must equal gbpt_render_device's (which uses the
context's growable buffers) on the same inputs: the per-path arithmetic and the per-pixel sample
order are the same, so the outputs are compared bit for bit, on two calls in a row (the array keeps
the previous call's contents). This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(native):
    import torch
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    ctx = S.Context(0)
    sc = S.cornell()
    sid = ctx.upload(sc)
    cam = S.workload_camera("cornell-256-16spp")
    yield ctx, sid, cam, N, S, torch
    ctx.destroy_scene(sid)
    ctx.close()


def _render_both(ctx, sid, cam, N, S, torch, params, n_pix):
    ref = torch.zeros((n_pix, 4), dtype=torch.float32, device="cuda")
    ctx.render_device(sid, cam, params, ref.data_ptr())
    ctx.synchronize()
    outs = []
    for _ in range(2):  # two calls in a row share the static array
        out = torch.full((n_pix, 4), -1.0, dtype=torch.float32, device="cuda")
        N.check(ctx.lib.gbpt_render_device_noalloc(ctx.handle, sid, C.byref(cam), C.byref(params),
                                                   out.data_ptr()))
        outs.append(out.cpu().numpy())
    return ref.cpu().numpy(), outs


@pytest.mark.parametrize("nee,rr,spp", [(False, 0, 16), (True, 3, 64)])
def test_noalloc_matches_render_device(setup, nee, rr, spp):
    ctx, sid, cam, N, S, torch = setup
    # 256 x 256 x 64 spp = 4.2M paths: the static array renders it in ~18 waves
    params, _ = S.render_params(256, 256, spp, 5, nee=nee, rr_depth=rr, frame=21)
    ref, outs = _render_both(ctx, sid, cam, N, S, torch, params, 256 * 256)
    assert np.all(np.isfinite(ref)) and ref[:, :3].max() > 0
    for out in outs:
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_noalloc_pixel_subset(setup):
    ctx, sid, cam, N, S, torch = setup
    pix = np.arange(3, 65536, 7, dtype=np.uint32)
    params, keep = S.render_params(256, 256, 32, 5, pixels=pix, frame=4)
    ref, outs = _render_both(ctx, sid, cam, N, S, torch, params, len(pix))
    for out in outs:
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_noalloc_rejects_oversize(setup):
    ctx, sid, cam, N, S, torch = setup
    out = torch.zeros((16, 4), dtype=torch.float32, device="cuda")
    params, _ = S.render_params(4, 4, 1 << 20, 5)  # spp beyond one pass over the array
    rc = ctx.lib.gbpt_render_device_noalloc(ctx.handle, sid, C.byref(cam), C.byref(params),
                                            out.data_ptr())
    assert rc == N.GBPT_ERR_INVALID
    assert b"exceeds" in ctx.lib.gbpt_last_error()

"""GPU tests of batched rendering and the request server.

A request's pixels are rendered within one tick from their own (pixel, frame, sample) seeds and
each pixel's samples are summed in a fixed order, so a request must give the same bits alone
(gbpt_render) and in any batch or server mix: every comparison here is bit-exact. The batches mix
scenes, resolutions, spp, path lengths, estimators, pixel lists and host/device outputs, and some
are sized so that requests span several ticks or share one.
"""
import ctypes as C
import threading
import time

import numpy as np
import pytest

from merian_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes(gpu_ctx):
    from merian_gb300 import scene as S
    corn = gpu_ctx.upload(S.cornell())
    soup = gpu_ctx.upload(S.soup(S.BASE_SEED, 200_000, 256, (256, 128)))
    cams = {
        corn: S.workload_camera("cornell-256-16spp"),
        soup: S.look_at((0.5, 0.5, -1.2), (0.5, 0.5, 0.5), (0, 1, 0), 45.0, 16 / 9),
    }
    yield corn, soup, cams
    gpu_ctx.destroy_scene(corn)
    gpu_ctx.destroy_scene(soup)


def _jobs(scenes, S):
    """A mixed set of requests: (scene, camera, params, pixel-list keepalive)."""
    corn, soup, cams = scenes
    rng = np.random.default_rng(7)
    jobs = []
    spec = [
        (corn, 64, 64, 16, 5, False, 0, None),
        (soup, 160, 90, 8, 8, True, 3, None),
        (corn, 128, 128, 1, 5, True, 0, None),
        (soup, 96, 54, 33, 4, False, 2, None),
        (corn, 256, 256, 4, 3, True, 3, rng.choice(65536, 3000, replace=False)),
        (soup, 320, 180, 2, 8, True, 3, rng.choice(320 * 180, 500, replace=False)),
        (corn, 32, 32, 0, 5, False, 0, None),  # no samples: zeros
        (soup, 48, 27, 64, 1, False, 0, None),  # primary emission only
    ]
    for i, (sid, w, h, spp, L, nee, rr, pix) in enumerate(spec):
        cam = cams[sid]
        if pix is not None:
            pix = np.sort(pix).astype(np.uint32)
        params, keep = S.render_params(w, h, spp, L, nee=nee, rr_depth=rr, frame=100 + i,
                                       pixels=pix)
        jobs.append((sid, cam, params, keep))
    return jobs


def _alone(gpu_ctx, jobs):
    return [gpu_ctx.render(sid, cam, p) for sid, cam, p, _ in jobs]


def _same(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_batch_equals_alone(gpu_ctx, scenes):
    from merian_gb300 import scene as S
    jobs = _jobs(scenes, S)
    ref = _alone(gpu_ctx, jobs)
    assert np.all(ref[6] == 0) and ref[1][:, :3].max() > 0
    outs, st = gpu_ctx.render_batch([(s, c, p) for s, c, p, _ in jobs], stats=True)
    for i, (a, b) in enumerate(zip(ref, outs)):
        assert _same(a, b), f"request {i} differs in the batch"
    assert st.samples == sum(len(r) * j[2].spp for r, j in zip(ref, jobs))
    # the same batch in reverse order
    outs = gpu_ctx.render_batch([(s, c, p) for s, c, p, _ in jobs][::-1])[::-1]
    for a, b in zip(ref, outs):
        assert _same(a, b)


def test_batch_with_graphs_equals_alone(gpu_ctx, scenes):
    from merian_gb300 import scene as S
    jobs = _jobs(scenes, S)
    ref = _alone(gpu_ctx, jobs)
    gpu_ctx.set_graphs(True)
    try:
        for _ in range(2):  # the second pass replays the captured graphs
            outs = gpu_ctx.render_batch([(s, c, p) for s, c, p, _ in jobs])
            for a, b in zip(ref, outs):
                assert _same(a, b)
    finally:
        gpu_ctx.set_graphs(False)


def test_batch_device_outputs(gpu_ctx, scenes):
    import torch
    from merian_gb300 import scene as S
    jobs = _jobs(scenes, S)[:4]
    ref = _alone(gpu_ctx, jobs)
    bufs = [torch.full((len(r), 4), -1.0, device="cuda") for r in ref]
    reqs = (N.Request * len(jobs))()
    for i, (sid, cam, p, _) in enumerate(jobs):
        reqs[i] = gpu_ctx.request(sid, cam, p, out_device=bufs[i].data_ptr())
    N.check(gpu_ctx.lib.gbpt_render_batch(gpu_ctx.handle, reqs, len(jobs), None))
    for a, b in zip(ref, bufs):
        assert _same(a, b.cpu().numpy())


def test_request_spanning_ticks(gpu_ctx, scenes):
    """512 x 512 x 40 spp = 10.5M paths: more than one 8 Mi-path tick, split by whole pixels."""
    from merian_gb300 import scene as S
    corn, soup, cams = scenes
    big, _ = S.render_params(512, 512, 40, 3, nee=True, frame=5)
    small, _ = S.render_params(64, 64, 16, 5, frame=6)
    ref_big = gpu_ctx.render(corn, cams[corn], big)
    ref_small = gpu_ctx.render(soup, cams[soup], small)
    outs = gpu_ctx.render_batch([(corn, cams[corn], big), (soup, cams[soup], small)])
    assert _same(ref_big, outs[0]) and _same(ref_small, outs[1])


def test_batch_rejects_bad_requests(gpu_ctx, scenes):
    from merian_gb300 import scene as S
    corn, soup, cams = scenes
    p, _ = S.render_params(16, 16, 1, 2)
    reqs = (N.Request * 1)()
    reqs[0] = gpu_ctx.request(corn, cams[corn], p)  # no output at all
    assert gpu_ctx.lib.gbpt_render_batch(gpu_ctx.handle, reqs, 1, None) == N.GBPT_ERR_INVALID
    out = np.zeros((256, 4), np.float32)
    reqs[0] = gpu_ctx.request(12345, cams[corn], p, out_host=out)
    assert gpu_ctx.lib.gbpt_render_batch(gpu_ctx.handle, reqs, 1, None) == N.GBPT_ERR_NOT_FOUND
    assert gpu_ctx.lib.gbpt_render_batch(gpu_ctx.handle, reqs, 0, None) == 0


# ---- the request server ------------------------------------------------------------------------

@pytest.fixture()
def server(gpu_ctx):
    started = []

    def start(**kw):
        gpu_ctx.server_start(**kw)
        started.append(True)
        return gpu_ctx

    yield start
    if started:
        gpu_ctx.server_stop()


@pytest.mark.parametrize("wave,graphs", [(0, False), (1 << 16, False), (1 << 16, True)])
def test_server_results_equal_alone(gpu_ctx, scenes, server, wave, graphs):
    """Each result is the same alone and in the mix: requests submitted together (and, with a
    64 Ki-path wave, split over many ticks shared with other requests)."""
    from merian_gb300 import scene as S
    jobs = _jobs(scenes, S)
    ref = _alone(gpu_ctx, jobs)
    ctx = server(wave_paths=wave, use_graphs=graphs)
    outs = [np.full_like(r, -1.0) for r in ref]
    tickets = [ctx.submit(s, c, p, out_host=o) for (s, c, p, _), o in zip(jobs, outs)]
    for t in tickets:
        rc, st = ctx.wait(t, 120.0)
        assert rc == 0 and st.state == N.REQ_DONE
        assert st.submit_s <= st.admit_s <= st.done_s
    for i, (a, b) in enumerate(zip(ref, outs)):
        assert _same(a, b), f"request {i} differs when served"
    info = ctx.server_info()
    assert info["completed"] >= len(jobs) and info["ticks"] >= 1
    if wave:  # small waves: the requests were spread over (at least) this many ticks
        paths = sum(len(r) * p.spp for r, (_, _, p, _) in zip(ref, jobs))
        assert info["ticks"] >= -(-paths // wave)
    for t in tickets:
        ctx.release(t)


def test_server_continuous_arrivals(gpu_ctx, scenes, server):
    """Requests submitted from another thread while earlier ones run join later ticks."""
    from merian_gb300 import scene as S
    jobs = _jobs(scenes, S)
    ref = _alone(gpu_ctx, jobs)
    ctx = server(wave_paths=1 << 18)
    outs = [np.full_like(r, -1.0) for r in ref]
    tickets = [None] * len(jobs)

    def client():
        for i, (s, c, p, _) in enumerate(jobs):
            tickets[i] = ctx.submit(s, c, p, out_host=outs[i])
            time.sleep(0.002)

    th = threading.Thread(target=client)
    th.start()
    th.join()
    for t in tickets:
        rc, st = ctx.wait(t, 120.0)
        assert rc == 0
    for a, b in zip(ref, outs):
        assert _same(a, b)


def test_server_cancel_and_busy_scene(gpu_ctx, scenes, server):
    from merian_gb300 import scene as S
    corn, soup, cams = scenes
    ctx = server(wave_paths=1 << 16, max_active=1)
    big, _ = S.render_params(256, 256, 64, 5, frame=1)
    out_a = np.zeros((256 * 256, 4), np.float32)
    out_b = np.zeros_like(out_a)
    ta = ctx.submit(corn, cams[corn], big, out_host=out_a)
    tb = ctx.submit(corn, cams[corn], big, out_host=out_b)  # waits behind ta (max_active = 1)
    # the scene is held by queued/running requests
    assert ctx.lib.gbpt_scene_destroy(ctx.handle, corn) == N.GBPT_ERR_BUSY
    ctx.cancel(tb)
    rc, st = ctx.wait(tb, 60.0)
    assert rc == N.GBPT_ERR_CANCELLED and st.state == N.REQ_CANCELLED
    ctx.cancel(ta)  # running: stops at a tick boundary
    rc, st = ctx.wait(ta, 60.0)
    assert st.state in (N.REQ_CANCELLED, N.REQ_DONE)
    assert ctx.lib.gbpt_server_poll(ctx.handle, 999999, None) == N.GBPT_ERR_NOT_FOUND


def test_server_stop_cancels_queued(gpu_ctx, scenes):
    from merian_gb300 import scene as S
    corn, soup, cams = scenes
    gpu_ctx.server_start(wave_paths=1 << 16, max_active=1)
    p, _ = S.render_params(256, 256, 32, 5, frame=2)
    outs = [np.zeros((256 * 256, 4), np.float32) for _ in range(3)]
    ts = [gpu_ctx.submit(corn, cams[corn], p, out_host=o) for o in outs]
    gpu_ctx.server_stop()
    # the scene is free again once the server is gone
    assert gpu_ctx.lib.gbpt_server_poll(gpu_ctx.handle, ts[0], None) == N.GBPT_ERR_INVALID
    sid = gpu_ctx.upload(S.cornell())
    gpu_ctx.destroy_scene(sid)


def test_material_sorted_shading_same_result(gpu_ctx, scenes):
    """'shader execution reordering' (sort_materials) only changes the order in which queue
    entries are shaded: every output is bit-identical, alone and in a batch."""
    from merian_gb300 import scene as S
    jobs = _jobs(scenes, S)
    ref = _alone(gpu_ctx, jobs)
    for _, _, p, _ in jobs:
        p.sort_materials = 1
    assert all(_same(a, b) for a, b in zip(ref, _alone(gpu_ctx, jobs)))
    outs = gpu_ctx.render_batch([(s, c, p) for s, c, p, _ in jobs])
    assert all(_same(a, b) for a, b in zip(ref, outs))


def test_tuning_and_autotune_same_result(gpu_ctx, scenes):
    """The context's tuning (tick size, forced material sort, graphs, two tick streams, the
    traversal's refill and postponement thresholds and blocks per SM) and the autotuner's choice
    change only the schedule: every output is bit-identical to the default schedule's."""
    from merian_gb300 import scene as S
    jobs = _jobs(scenes, S)
    ref = _alone(gpu_ctx, jobs)
    corn, soup, cams = scenes
    try:
        for wave, sort, graphs, streams, refill, postpone, bps in (
                (1 << 12, 1, False, 2, 0, 0, 0), (1 << 20, 0, True, 0, 32, 1, 1),
                (1 << 24, -1, False, 2, 1, 32, 3), (1 << 16, 0, False, 2, 12, 12, 7),
                (1 << 22, 1, True, 1, 28, 2, 64)):
            gpu_ctx.set_tuning(wave, sort, graphs, streams=streams, refill_lanes=refill,
                               postpone_lanes=postpone, blocks_per_sm=bps)
            t = gpu_ctx.get_tuning()
            assert (t.wave_paths, t.sort_materials, t.use_graphs, t.streams) == \
                (wave, sort, int(graphs), streams)
            assert (t.trace_refill_lanes, t.trace_postpone_lanes, t.trace_blocks_per_sm) == \
                (refill, postpone, bps)
            assert all(_same(a, b) for a, b in zip(ref, _alone(gpu_ctx, jobs)))
            outs = gpu_ctx.render_batch([(s, c, p) for s, c, p, _ in jobs if p.spp <= wave])
            kept = [r for r, j in zip(ref, jobs) if j[2].spp <= wave]
            assert all(_same(a, b) for a, b in zip(kept, outs))
        with pytest.raises(N.GbptError):
            gpu_ctx.set_tuning(100, 0, False)  # below the smallest tick
        with pytest.raises(N.GbptError):
            gpu_ctx.set_tuning(1 << 20, 0, False, streams=3)
        with pytest.raises(N.GbptError):
            gpu_ctx.set_tuning(1 << 20, 0, False, refill_lanes=33)
        with pytest.raises(N.GbptError):
            gpu_ctx.set_tuning(1 << 20, 0, False, blocks_per_sm=-1)
        gpu_ctx.set_tuning(0, -1, False)
        p, _ = S.render_params(320, 180, 16, 8, nee=True, rr_depth=3, frame=1)
        t, ms = gpu_ctx.autotune(soup, cams[soup], p)
        # 8 tick size x sorting candidates, 5 refill, 5 postponement, 3 blocks-per-SM candidates
        assert len(ms) == 21 and all(m > 0 for m in ms)
        assert t.wave_paths in (1 << 21, 1 << 22, 1 << 23, 1 << 24) and t.sort_materials in (0, 1)
        assert t.trace_refill_lanes in (12, 16, 20, 24, 28)
        assert t.trace_postpone_lanes in (2, 4, 6, 8, 12)
        assert t.trace_blocks_per_sm in (6, 7, 0)
        got = gpu_ctx.get_tuning()
        assert (got.wave_paths, got.sort_materials, got.trace_refill_lanes,
                got.trace_postpone_lanes, got.trace_blocks_per_sm) == \
            (t.wave_paths, t.sort_materials, t.trace_refill_lanes, t.trace_postpone_lanes,
             t.trace_blocks_per_sm)
        assert all(_same(a, b) for a, b in zip(ref, _alone(gpu_ctx, jobs)))
        # the same bucket again: the cached result, no candidate rendered again
        gpu_ctx.set_tuning(0, -1, False)
        t2, ms2 = gpu_ctx.autotune(soup, cams[soup], p)
        assert bytes(t2) == bytes(t) and ms2 == ms
    finally:
        gpu_ctx.set_tuning(0, -1, False)

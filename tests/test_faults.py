"""Failure handling without a GPU fault: device allocations refused on the host side
(gbpt_debug_fail_allocations) during scene creation and rendering must return
GBPT_ERR_NO_MEMORY, free what the call had allocated and leave the context usable; the next
call gives the same bits as a context that never failed.

CPU: the injection's argument checks. GPU: every allocation of a scene upload and of a first
render failed in turn.
"""
import numpy as np
import pytest


def test_injection_arguments(native):
    from merian_gb300 import _native as N
    lib = N.load()
    assert lib.gbpt_debug_fail_allocations(-1, 1) == N.GBPT_ERR_INVALID
    assert lib.gbpt_debug_fail_allocations(0, -1) == N.GBPT_ERR_INVALID
    assert lib.gbpt_debug_fail_allocations(3, 2) == N.GBPT_OK
    assert lib.gbpt_debug_fail_allocations(0, 0) == N.GBPT_OK


@pytest.mark.gpu
def test_injected_allocation_failures(gpu_ctx):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    lib = gpu_ctx.lib
    sc = S.cornell()
    cam = S.workload_camera("cornell-256-16spp")
    p, _ = S.render_params(64, 64, 4, 5, nee=True, rr_depth=3, frame=1)
    sid = gpu_ctx.upload(sc)
    ref = gpu_ctx.render(sid, cam, p)
    gpu_ctx.destroy_scene(sid)
    with S.Context(0) as ctx:
        try:
            # scene creation: fail its k-th device allocation, k = 0, 1, ... until it succeeds
            ctx.synchronize()
            base = ctx.memory_info()["free"]
            failed = 0
            for k in range(64):
                N.check(lib.gbpt_debug_fail_allocations(k, 1))
                try:
                    sid = ctx.upload(sc)
                except N.GbptError as e:
                    assert e.code == N.GBPT_ERR_NO_MEMORY
                    failed += 1
                    continue
                break
            N.check(lib.gbpt_debug_fail_allocations(0, 0))
            assert failed >= 5  # BVH nodes, triangles, vertices, indices, geometries, ...
            ctx.destroy_scene(sid)
            ctx.synchronize()
            assert abs(ctx.memory_info()["free"] - base) <= (4 << 20)  # nothing leaked
            sid = ctx.upload(sc)
            # the first render of a context: tick tables, path state, queues, pixel cache and
            # the output staging buffer are allocated; fail each in turn
            failed = 0
            for k in range(64):
                N.check(lib.gbpt_debug_fail_allocations(k, 1))
                try:
                    out = ctx.render(sid, cam, p)
                except N.GbptError as e:
                    assert e.code == N.GBPT_ERR_NO_MEMORY
                    failed += 1
                    continue
                break
            N.check(lib.gbpt_debug_fail_allocations(0, 0))
            assert failed >= 10
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
            assert np.array_equal(ctx.render(sid, cam, p).view(np.uint32), ref.view(np.uint32))
            ctx.destroy_scene(sid)
        finally:
            lib.gbpt_debug_fail_allocations(0, 0)

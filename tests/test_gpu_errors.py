"""The kernels' error word, reached on purpose without a GPU fault.

A variant build of the library with a 2-entry traversal stack (GBPT_STACK_SIZE=2) makes the rays of
a deep scene overflow their stack. The overflow sets the error word of the tick's work buffers and
finishes the ray with what it found; no kernel traps, faults or waits. The host must report it:
  * gbpt_render returns GBPT_ERR_DEVICE with the overflow named, also when only the ticks of the
    second tick stream overflow (a pixel list whose first tick sees only the sky, whose second sees
    the soup), and with one stream;
  * the request server fails the requests of the tick with GBPT_ERR_DEVICE;
  * the context stays usable: the flag is cleared, and a scene that never fills the stack renders
    the bits the default build gives.
"""
import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

W = H = 64


@pytest.fixture(scope="module")
def small_stack_lib(native):
    from merian_gb300 import _native as N
    from merian_gb300 import build as B
    out = ROOT / "merian_gb300" / "_build" / "stack2"
    lib = B.build(defines=("GBPT_STACK_SIZE=2",), lib=out / "libgbpt.so", build_dir=out)
    return N.load(lib)


def quad():
    """Two triangles facing the camera: the root's two leaf children, nothing ever pushed."""
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    v = np.zeros(4, N.VERTEX_DTYPE)
    v["position"] = [[-1, -1, 2], [1, -1, 2], [1, 1, 2], [-1, 1, 2]]
    g = np.zeros(1, N.GEOMETRY_DTYPE)
    g["triangle_count"] = 2
    g["flags"] = N.MESH_TWO_SIDED | N.MESH_FLAT_SHADING
    g["instance_mask"] = 0xFF
    m = np.zeros(1, N.MATERIAL_DTYPE)
    m["model"] = N.MATERIAL_DIFFUSE
    m["base_color"] = 0.6
    m["specular_alpha"] = 1.0
    m["specular_ior"] = 1.5
    m["base_color_texture"] = -1
    m["alpha_texture"] = -1
    env = np.full((8, 16, 4), 0.5, np.float32)
    return S.SceneData(v, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), g, m, env)


@pytest.fixture(scope="module")
def scenes():
    from merian_gb300 import scene as S
    soup = S.soup(S.BASE_SEED, 200_000, 256, (64, 32))
    # level with the soup's top face, looking along +z: the image's upper half looks up and away
    # from the unit cube (its rays miss the root box), the lower half down into the soup
    cam = S.look_at((0.5, 1.6, -1.5), (0.5, 1.6, 0.5), (0, 1, 0), 60.0, 1.0)
    return soup, cam, quad(), S.look_at((0, 0, 0), (0, 0, 1), (0, 1, 0), 60.0, 1.0)


def _params(spp, pixels):
    from merian_gb300 import scene as S
    return S.render_params(W, H, spp, 5, nee=True, rr_depth=3, frame=7, pixels=pixels)


def test_overflow_on_second_stream_is_reported(small_stack_lib, scenes):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    soup, cam, q, qcam = scenes
    top = np.arange(0, W * H // 2, dtype=np.uint32)
    bottom = np.arange(W * H // 2, W * H, dtype=np.uint32)
    with S.Context(0, lib=small_stack_lib) as ctx:
        sid, qid = ctx.upload(soup), ctx.upload(q)
        # the sky alone: no traversal ever pushes, no error
        p, keep = _params(1, top)
        sky = ctx.render(sid, cam, p)
        with S.Context(0) as ref:
            rsid = ref.upload(soup)
            assert np.array_equal(sky.view(np.uint32), ref.render(rsid, cam, p).view(np.uint32))
        # tick 0 (context stream): the sky; tick 1 (second stream): the soup, which overflows
        for streams in (0, 1):
            ctx.set_tuning(wave_paths=len(top), streams=streams)
            p, keep = _params(1, np.concatenate([top, bottom]))
            with pytest.raises(N.GbptError) as e:
                ctx.render(sid, cam, p)
            assert e.value.code == N.GBPT_ERR_DEVICE
            assert "stack overflow" in str(e.value)
            # the flag was cleared: a scene that never fills the stack renders clean
            pq, _ = S.render_params(W, H, 4, 5, nee=True, frame=3)
            a = ctx.render(qid, qcam, pq)
            with S.Context(0) as ref:
                b = ref.render(ref.upload(q), qcam, pq)
            assert np.all(np.isfinite(a))
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_overflow_fails_server_requests(small_stack_lib, scenes):
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    soup, cam, q, qcam = scenes
    with S.Context(0, lib=small_stack_lib) as ctx:
        sid, qid = ctx.upload(soup), ctx.upload(q)
        ctx.server_start(wave_paths=1 << 16)
        try:
            p, keep = _params(2, None)
            out = np.empty((W * H, 4), np.float32)
            t = ctx.submit(sid, cam, p, out_host=out)
            rc, st = ctx.wait(t, -1.0)
            assert rc == N.GBPT_ERR_DEVICE
            # a later request on a shallow scene completes
            pq, _ = S.render_params(W, H, 2, 5, frame=1)
            out2 = np.empty((W * H, 4), np.float32)
            rc2, _ = ctx.wait(ctx.submit(qid, qcam, pq, out_host=out2), -1.0)
            assert rc2 == N.GBPT_OK and np.all(np.isfinite(out2))
        finally:
            ctx.server_stop()

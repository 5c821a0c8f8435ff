"""Scene data, the device context and the benchmark workloads.

``SceneData`` holds the host arrays of one scene in the layouts of ``include/gbpt.h`` (merian's
PackedVertexData / GeometryData / material records). ``Context`` owns a ``gbpt_ctx``: scenes
uploaded to HBM and the render / traversal entry points.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

BASE_SEED = 0x1234567


@dataclass
class SceneData:
    vertices: np.ndarray
    indices: np.ndarray
    geometries: np.ndarray
    materials: np.ndarray
    env: np.ndarray | None = None          # (h, w, 4) float32
    env_to_local: np.ndarray = field(default_factory=lambda: np.eye(3, dtype=np.float32))
    env_intensity: float = 1.0
    # two-level scenes: BLAS geometry ranges (BLAS_DTYPE) and instances (INSTANCE_DTYPE)
    blas_ranges: np.ndarray | None = None
    instances: np.ndarray | None = None
    # RGBA8 textures: (height, width, 4) uint8 arrays and whether each is sRGB-encoded
    textures: list = field(default_factory=list)

    @property
    def triangle_count(self) -> int:
        return int(self.indices.shape[0])

    def desc(self):
        """(SceneDesc, keep-alive objects) for gbpt_scene_create / the oracle."""
        keep = []
        env_p = None
        if self.env is not None:
            env = np.ascontiguousarray(self.env, dtype=np.float32)
            keep.append(env)
            e = N.EnvMap()
            e.texels = env.ctypes.data_as(C.POINTER(C.c_float))
            e.height, e.width = int(env.shape[0]), int(env.shape[1])
            e.to_local[:] = [float(x) for x in np.asarray(self.env_to_local, np.float32).reshape(9)]
            e.intensity = float(self.env_intensity)
            keep.append(e)
            env_p = C.pointer(e)
        d = N.SceneDesc()
        d.vertices = N.ptr(self.vertices)
        d.vertex_count = len(self.vertices)
        d.indices = N.ptr(self.indices)
        d.triangle_count = self.triangle_count
        d.geometries = N.ptr(self.geometries)
        d.geometry_count = len(self.geometries)
        d.materials = N.ptr(self.materials)
        d.material_count = len(self.materials)
        d.env = env_p
        if self.textures:
            arr = (N.Texture * len(self.textures))()
            for i, (tex, srgb) in enumerate(self.textures):
                t = np.ascontiguousarray(tex, dtype=np.uint8)
                keep.append(t)
                arr[i].texels = t.ctypes.data_as(C.POINTER(C.c_uint8))
                arr[i].height, arr[i].width = int(t.shape[0]), int(t.shape[1])
                arr[i].srgb = int(bool(srgb))
            keep.append(arr)
            d.textures = C.cast(arr, C.POINTER(N.Texture))
            d.texture_count = len(self.textures)
        if self.instances is not None and len(self.instances):
            b = np.ascontiguousarray(self.blas_ranges, dtype=N.BLAS_DTYPE)
            ins = np.ascontiguousarray(self.instances, dtype=N.INSTANCE_DTYPE)
            keep += [b, ins]
            d.blas_ranges = N.ptr(b)
            d.blas_count = len(b)
            d.instances = N.ptr(ins)
            d.instance_count = len(ins)
        return d, keep


def _gen_check(lib, rc: int, what: str) -> None:
    if rc != N.GBPT_OK:
        raise N.GbptError(rc, f"{what} failed")


def cornell(seed: int = BASE_SEED, tess: int = 1, lib=None) -> SceneData:
    """The Cornell box: 1,024 triangles (gbpt_gen_cornell), or every grid refined `tess` times per
    side, 1,024 tess^2 triangles (gbpt_gen_cornell_tess). `lib`: the library whose gbpt_gen_*
    to call (default libgbpt.so)."""
    lib = lib or N.load()
    nt = 1024 * tess * tess
    v = np.zeros(3 * nt, N.VERTEX_DTYPE)
    i = np.zeros((nt, 3), np.uint32)
    g = np.zeros(8, N.GEOMETRY_DTYPE)
    m = np.zeros(8, N.MATERIAL_DTYPE)
    if tess == 1:
        _gen_check(lib, lib.gbpt_gen_cornell(seed, N.ptr(v), N.ptr(i), N.ptr(g), N.ptr(m)),
                   "gbpt_gen_cornell")
    else:
        _gen_check(lib, lib.gbpt_gen_cornell_tess(seed, tess, N.ptr(v), N.ptr(i), N.ptr(g),
                                                  N.ptr(m)), "gbpt_gen_cornell_tess")
    return SceneData(v, i, g, m)


def blob(seed: int, n_u: int = 250, n_v: int = 101):
    """(vertices, indices) of a bumpy closed sphere (gbpt_gen_blob), 2 n_u (n_v - 1) triangles."""
    lib = N.load()
    v = np.zeros((n_u + 1) * n_v, N.VERTEX_DTYPE)
    i = np.zeros((2 * n_u * (n_v - 1), 3), np.uint32)
    N.check(lib.gbpt_gen_blob(seed, n_u, n_v, N.ptr(v), N.ptr(i)))
    return v, i


def noise_texture(seed: int, width: int = 512, height: int = 512) -> np.ndarray:
    lib = N.load()
    t = np.zeros((height, width, 4), np.uint8)
    N.check(lib.gbpt_gen_noise_texture(seed, width, height, N.ptr(t)))
    return t


def env_lobes(seed: int, width: int = 2048, height: int = 1024, lib=None) -> np.ndarray:
    lib = lib or N.load()
    t = np.zeros((height, width, 4), np.float32)
    _gen_check(lib, lib.gbpt_gen_env(seed, width, height, N.ptr(t)), "gbpt_gen_env")
    return t


def soup(seed: int = BASE_SEED, n_triangles: int = 1_000_000, n_geometries: int = 4096,
         env_size: tuple[int, int] | None = (2048, 1024), lib=None) -> SceneData:
    """Triangle soup with an optional Gaussian-lobe lat-long environment (gbpt_gen_soup)."""
    lib = lib or N.load()
    n_geometries = max(1, min(n_geometries, n_triangles))
    v = np.zeros(3 * n_triangles, N.VERTEX_DTYPE)
    i = np.zeros((n_triangles, 3), np.uint32)
    g = np.zeros(n_geometries, N.GEOMETRY_DTYPE)
    m = np.zeros(n_geometries, N.MATERIAL_DTYPE)
    _gen_check(lib, lib.gbpt_gen_soup(seed, n_triangles, n_geometries, N.ptr(v), N.ptr(i),
                                      N.ptr(g), N.ptr(m)), "gbpt_gen_soup")
    env = env_lobes(seed ^ 0xE27, *env_size, lib=lib) if env_size else None
    return SceneData(v, i, g, m, env)


def build_bvh(scene: SceneData, bvh_build: int = N.BVH_SPLIT):
    """The traversal data gbpt_scene_create builds for `scene`, built on the host (gbpt_bvh_build,
    no device): (nodes (n, 80) uint8, triangle records (m, 48) uint8, depth)."""
    lib = N.load()
    d, keep = scene.desc()
    h = C.c_void_p()
    N.check(lib.gbpt_bvh_build(C.byref(d), bvh_build, C.byref(h)))
    try:
        np_, nn, tp, nt, dp = C.c_void_p(), C.c_uint64(), C.c_void_p(), C.c_uint64(), C.c_uint32()
        N.check(lib.gbpt_bvh_info(h, C.byref(np_), C.byref(nn), C.byref(tp), C.byref(nt),
                                  C.byref(dp)))
        nodes = np.ctypeslib.as_array((C.c_uint8 * (80 * nn.value)).from_address(np_.value)) \
            .reshape(-1, 80).copy() if nn.value else np.zeros((0, 80), np.uint8)
        tris = np.ctypeslib.as_array((C.c_uint8 * (48 * nt.value)).from_address(tp.value)) \
            .reshape(-1, 48).copy() if nt.value else np.zeros((0, 48), np.uint8)
        return nodes, tris, dp.value
    finally:
        lib.gbpt_bvh_free(h)


def look_at(position, target, up=(0.0, 1.0, 0.0), vfov_deg: float = 40.0, aspect: float = 1.0,
            near: float = 0.1, far: float = 1000.0) -> N.Camera:
    """merian Camera basis (camera.cpp:263-266,349-367); near/far are merian's defaults."""
    lib = N.load()
    cam = N.Camera()
    f3 = C.c_float * 3
    N.check(lib.gbpt_camera_look_at(f3(*position), f3(*target), f3(*up),
                                    math.radians(vfov_deg), aspect, near, far, C.byref(cam)))
    return cam


def render_params(width: int, height: int, spp: int, max_path_length: int, *,
                  emission_on_primary: bool = True, instance_mask: int = 0xFF,
                  frame: int = 0, nee: bool = False, rr_depth: int = 0,
                  sort_materials: bool = False, demodulate_albedo: bool = False,
                  pixels: np.ndarray | None = None):
    p = N.RenderParams()
    p.width, p.height, p.spp, p.max_path_length = width, height, spp, max_path_length
    p.emission_on_primary = int(emission_on_primary)
    p.instance_mask = instance_mask
    p.frame = frame
    p.nee = int(nee)
    p.rr_depth = rr_depth
    p.sort_materials = int(sort_materials)
    p.demodulate_albedo = int(demodulate_albedo)
    keep = None
    if pixels is not None and len(pixels):
        keep = np.ascontiguousarray(pixels, dtype=np.uint32)
        p.pixels = keep.ctypes.data_as(C.POINTER(C.c_uint32))
        p.pixel_count = len(keep)
    return p, keep


# ---- the benchmark workloads -------------------------------------------------------------------
WORKLOADS = {
    # strict-parity configuration: the reference's BSDF-only estimator
    "cornell-256-16spp": dict(scene="cornell", width=256, height=256, spp=16, max_path_length=5,
                              nee=False, rr_depth=0,
                              camera=dict(position=(0.5, 0.5, -1.4), target=(0.5, 0.5, 0.0),
                                          vfov_deg=40.0)),
    # the headline: 1M-triangle soup, 1080p, 64 spp, path length 8, NEE + roulette from depth 3
    "soup-1m-1080p-64spp": dict(scene="soup", n_triangles=1_000_000, width=1920, height=1080,
                                spp=64, max_path_length=8, nee=True, rr_depth=3,
                                # the whole 16:9 frame sees the soup's front face
                                camera=dict(position=(0.5, 0.5, -0.6), target=(0.5, 0.5, 0.5),
                                            vfov_deg=45.0)),
    # the same scene and estimator on a smaller frame: the case the ncu captures run on
    "soup-1m-360p-16spp": dict(scene="soup", n_triangles=1_000_000, width=640, height=360,
                               spp=16, max_path_length=8, nee=True, rr_depth=3,
                               camera=dict(position=(0.5, 0.5, -0.6), target=(0.5, 0.5, 0.5),
                                           vfov_deg=45.0)),
}


def load_pbrt(path: str):
    """A pbrt-v4 scene file through gbpt_load_pbrt: (SceneData with its own copies of the arrays,
    the file's camera, (width, height), warnings)."""
    return _load_file("gbpt_load_pbrt", path)


def load_gltf(path: str):
    """A glTF 2.0 file (.gltf / .glb) through gbpt_load_gltf; returns like load_pbrt."""
    return _load_file("gbpt_load_gltf", path)


def _load_file(entry: str, path: str):
    lib = N.load()
    h = C.c_void_p()
    N.check(getattr(lib, entry)(str(path).encode(), C.byref(h)))
    try:
        info = N.LoadedInfo()
        N.check(lib.gbpt_loaded_scene_info(h, C.byref(info)))
        d = info.desc

        def arr(ptr, n, dtype):
            if not n:
                return np.zeros(0, dtype)
            buf = (C.c_uint8 * (n * dtype.itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype).copy()

        verts = arr(d.vertices, d.vertex_count, N.VERTEX_DTYPE)
        idx = arr(d.indices, 3 * d.triangle_count, np.dtype(np.uint32)).reshape(-1, 3)
        geoms = arr(d.geometries, d.geometry_count, N.GEOMETRY_DTYPE)
        mats = arr(d.materials, d.material_count, N.MATERIAL_DTYPE)
        env = None
        intensity = 1.0
        if d.env:
            e = d.env.contents
            env = np.ctypeslib.as_array(e.texels, (e.height, e.width, 4)).copy()
            intensity = float(e.intensity)
        blas = inst = None
        if d.instance_count:
            blas = arr(d.blas_ranges, d.blas_count, N.BLAS_DTYPE)
            inst = arr(d.instances, d.instance_count, N.INSTANCE_DTYPE)
        warnings = [lib.gbpt_loaded_scene_warning(h, i).decode()
                    for i in range(info.warning_count)]
        textures = []
        for t in range(d.texture_count):
            tx = d.textures[t]
            px = np.ctypeslib.as_array(tx.texels, (tx.height, tx.width, 4)).copy()
            textures.append((px, bool(tx.srgb)))
        cam = N.Camera.from_buffer_copy(info.camera)
        sc = SceneData(verts, idx, geoms, mats, env, env_intensity=intensity, blas_ranges=blas,
                       instances=inst, textures=textures)
        return sc, cam, (int(info.width), int(info.height)), warnings
    finally:
        lib.gbpt_loaded_scene_free(h)


def workload_scene(name: str, seed: int = BASE_SEED, lib=None, **overrides) -> SceneData:
    w = dict(WORKLOADS[name], **overrides)
    if w["scene"] == "cornell":
        return cornell(seed, lib=lib)
    return soup(seed, w.get("n_triangles", 1_000_000), w.get("n_geometries", 4096),
                w.get("env_size", (2048, 1024)), lib=lib)


def workload_camera(name: str, width: int | None = None, height: int | None = None) -> N.Camera:
    w = WORKLOADS[name]
    width = width or w["width"]
    height = height or w["height"]
    c = w["camera"]
    return look_at(c["position"], c["target"], (0.0, 1.0, 0.0), c["vfov_deg"], width / height)


class Context:
    """One gbpt_ctx on one CUDA device; scenes stay resident in HBM until destroyed."""

    def __init__(self, device: int = 0, stream: int = 0, lib=None):
        """`lib`: a build of the library loaded with _native.load(path) (a variant with other
        compile-time constants); default libgbpt.so."""
        self.lib = lib or N.load()
        h = C.c_void_p()
        self._check(self.lib.gbpt_create(device, stream, C.byref(h)))
        self.handle = h

    def _check(self, rc: int) -> None:
        if rc != N.GBPT_OK:
            msg = self.lib.gbpt_last_error()
            raise N.GbptError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if self.handle:
            self.lib.gbpt_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload(self, scene: SceneData) -> int:
        d, keep = scene.desc()
        sid = C.c_uint32()
        self._check(self.lib.gbpt_scene_create(self.handle, C.byref(d), C.byref(sid)))
        del keep
        return sid.value

    def destroy_scene(self, sid: int) -> None:
        self._check(self.lib.gbpt_scene_destroy(self.handle, sid))

    def scene_stats(self, sid: int) -> dict:
        n, t, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
        dp = C.c_uint32()
        self._check(self.lib.gbpt_scene_stats(self.handle, sid, C.byref(n), C.byref(t), C.byref(b),
                                          C.byref(dp)))
        return dict(nodes=n.value, tris=t.value, bytes=b.value, depth=dp.value)

    def render(self, sid: int, camera: N.Camera, params: N.RenderParams,
               stats: bool = False):
        n = params.pixel_count or params.width * params.height
        out = np.empty((n, 4), np.float32)
        st = N.RenderStats()
        self._check(self.lib.gbpt_render(self.handle, sid, C.byref(camera), C.byref(params),
                                     N.ptr(out), C.byref(st) if stats else None))
        return (out, st) if stats else out

    def render_device(self, sid: int, camera: N.Camera, params: N.RenderParams, out_ptr: int,
                      stats: bool = False):
        st = N.RenderStats()
        self._check(self.lib.gbpt_render_device(self.handle, sid, C.byref(camera), C.byref(params),
                                            out_ptr, C.byref(st) if stats else None))
        return st if stats else None

    def trace_primary(self, sid: int, camera: N.Camera, width: int, height: int,
                      mask: int = 0xFF) -> np.ndarray:
        hits = np.zeros(width * height, N.HIT_DTYPE)
        self._check(self.lib.gbpt_trace_primary(self.handle, sid, C.byref(camera), width, height, mask,
                                            N.ptr(hits)))
        return hits

    def trace(self, sid: int, rays_dev: int, n: int, hits_dev: int, mask: int = 0xFF,
              any_hit: bool = False, counted: bool = False):
        if counted:
            a, b = C.c_double(), C.c_double()
            self._check(self.lib.gbpt_trace_counted(self.handle, sid, rays_dev, n, mask, int(any_hit),
                                                hits_dev, C.byref(a), C.byref(b)))
            return a.value, b.value
        self._check(self.lib.gbpt_trace(self.handle, sid, rays_dev, n, mask, int(any_hit), hits_dev))
        return None

    def synchronize(self) -> None:
        self._check(self.lib.gbpt_synchronize(self.handle))

    def set_profiling(self, level: int) -> None:
        self._check(self.lib.gbpt_set_profiling(self.handle, level))

    def memory_info(self) -> dict:
        f, t, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self.lib.gbpt_memory_info(self.handle, C.byref(f), C.byref(t), C.byref(c)))
        return dict(free=f.value, total=t.value, ctx=c.value)

    # ---- batches and the request server ----------------------------------------------------
    @staticmethod
    def request(sid: int, camera: N.Camera, params: N.RenderParams, out_host: np.ndarray | None = None,
                out_device: int | None = None) -> N.Request:
        r = N.Request()
        r.scene = sid
        r.camera = camera
        r.params = params
        r.out_host = N.ptr(out_host) if out_host is not None else None
        r.out_device = out_device
        return r

    def render_batch(self, jobs, stats: bool = False):
        """jobs: (scene id, camera, params) triples; returns one (n, 4) float32 array per job."""
        outs, reqs = [], (N.Request * max(len(jobs), 1))()
        for i, (sid, cam, params) in enumerate(jobs):
            n = params.pixel_count or params.width * params.height
            outs.append(np.empty((n, 4), np.float32))
            reqs[i] = self.request(sid, cam, params, out_host=outs[-1])
        st = N.RenderStats()
        self._check(self.lib.gbpt_render_batch(self.handle, reqs, len(jobs),
                                           C.byref(st) if stats else None))
        return (outs, st) if stats else outs

    def set_graphs(self, enable: bool) -> None:
        self._check(self.lib.gbpt_set_graphs(self.handle, int(enable)))

    def set_tuning(self, wave_paths: int = 0, sort_materials: int = -1,
                   use_graphs: bool = False, bvh_build: int = N.BVH_SPLIT,
                   streams: int = 0, refill_lanes: int = 0, postpone_lanes: int = 0,
                   blocks_per_sm: int = 0) -> None:
        t = N.Tuning(wave_paths, sort_materials, int(use_graphs), bvh_build, streams,
                     refill_lanes, postpone_lanes, blocks_per_sm)
        self._check(self.lib.gbpt_set_tuning(self.handle, C.byref(t)))

    def get_tuning(self) -> N.Tuning:
        t = N.Tuning()
        self._check(self.lib.gbpt_get_tuning(self.handle, C.byref(t)))
        return t

    def autotune(self, sid: int, camera: N.Camera, params: N.RenderParams):
        """Times the candidate schedules on one frame and keeps the fastest; returns the chosen
        tuning and the candidates' times (ms, in gbpt_autotune's order; candidates not run are
        left out)."""
        t = N.Tuning()
        ms = (C.c_double * N.AUTOTUNE_CANDIDATES)(*([float("nan")] * N.AUTOTUNE_CANDIDATES))
        self._check(self.lib.gbpt_autotune(self.handle, sid, C.byref(camera), C.byref(params),
                                       C.byref(t), ms))
        return t, [v for v in ms if v == v]

    def clock(self) -> float:
        return self.lib.gbpt_clock()

    def server_start(self, wave_paths: int = 0, arena_bytes: int = 0, use_graphs: bool = False,
                     max_active: int = 0) -> None:
        cfg = N.ServerConfig(wave_paths, arena_bytes, int(use_graphs), max_active)
        self._check(self.lib.gbpt_server_start(self.handle, C.byref(cfg)))

    def server_stop(self) -> None:
        self._check(self.lib.gbpt_server_stop(self.handle))

    def submit(self, sid: int, camera: N.Camera, params: N.RenderParams,
               out_host: np.ndarray | None = None, out_device: int | None = None) -> int:
        """Queues a request; out_host (or the device buffer) must stay alive until it finishes."""
        t = C.c_uint64()
        r = self.request(sid, camera, params, out_host, out_device)
        self._check(self.lib.gbpt_server_submit(self.handle, C.byref(r), C.byref(t)))
        return t.value

    def poll(self, ticket: int) -> tuple[int, N.RequestStatus]:
        st = N.RequestStatus()
        rc = self.lib.gbpt_server_poll(self.handle, ticket, C.byref(st))
        return rc, st

    def wait(self, ticket: int, timeout_s: float = -1.0) -> tuple[int, N.RequestStatus]:
        st = N.RequestStatus()
        rc = self.lib.gbpt_server_wait(self.handle, ticket, timeout_s, C.byref(st))
        return rc, st

    def cancel(self, ticket: int) -> None:
        self._check(self.lib.gbpt_server_cancel(self.handle, ticket))

    def release(self, ticket: int) -> None:
        self._check(self.lib.gbpt_server_release(self.handle, ticket))

    def server_info(self) -> dict:
        st = N.ServerStats()
        self._check(self.lib.gbpt_server_info(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in N.ServerStats._fields_}

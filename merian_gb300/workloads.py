"""Seeded synthetic request mixes: the batched configuration (many independent scenes rendered
together) and the served stream (Poisson arrivals over resident scenes).

Scenes below 100k triangles are the Cornell box with its grids refined (gbpt_gen_cornell_tess,
tessellated walls and boxes as in the 1,024-triangle box); larger ones are the triangle soup of the
headline configuration with a 512x256 Gaussian-lobe environment. Every request uses the
estimator of its scene type: Cornell boxes path length 5, soups path length 8, both with NEE and
Russian roulette from depth 3.
"""
from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from . import _native as N
from . import scene as S

BATCH_RESOLUTIONS = ((256, 256), (512, 512), (1024, 1024))
SERVED_RESOLUTIONS = ((512, 512), (1024, 1024), (1920, 1080))
SERVED_SPP = (1, 4, 16, 64)
# small requests (previews, tiles, thumbnails): one alone leaves most of the GPU idle
SMALL_RESOLUTIONS = ((64, 64), (128, 128), (256, 256), (512, 512))
SMALL_SPP = (1, 2, 4)


@dataclass
class SceneSpec:
    kind: str  # "cornell" or "soup"
    triangles: int
    seed: int

    def build(self) -> S.SceneData:
        if self.kind == "cornell":
            tess = max(1, int(round(math.sqrt(self.triangles / 1024))))
            return S.cornell(self.seed, tess)
        n_geom = max(1, min(4096, self.triangles // 64))
        return S.soup(self.seed, self.triangles, n_geom, (512, 256))


@dataclass
class RequestSpec:
    scene: int  # index into the scene list
    width: int
    height: int
    spp: int
    frame: int
    arrival_s: float = 0.0
    upload: SceneSpec | None = None  # a request that brings its own new scene


def scene_spec(rng: np.random.Generator, lo: float, hi: float) -> SceneSpec:
    n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    kind = "cornell" if n < 100_000 else "soup"
    if kind == "cornell":  # the refined box has 1024 tess^2 triangles
        tess = max(1, int(round(math.sqrt(n / 1024))))
        n = 1024 * tess * tess
    return SceneSpec(kind, n, int(rng.integers(1 << 62)))


def camera(kind: str, width: int, height: int):
    if kind == "cornell":
        return S.look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.0), (0.0, 1.0, 0.0), 40.0, width / height)
    return S.look_at((0.5, 0.5, -0.6), (0.5, 0.5, 0.5), (0.0, 1.0, 0.0), 45.0, width / height)


def params(kind: str, req: RequestSpec):
    L = 5 if kind == "cornell" else 8
    p, _ = S.render_params(req.width, req.height, req.spp, L, nee=True, rr_depth=3,
                           frame=req.frame)
    return p


def batch_mix(seed: int = S.BASE_SEED, n: int = 256, tri_range=(1e3, 2e6)):
    """n independent scenes (triangles log-uniform in tri_range), one request each: resolution
    from {256^2, 512^2, 1024^2}, spp uniform in 1..64."""
    rng = np.random.default_rng(seed)
    scenes = [scene_spec(rng, *tri_range) for _ in range(n)]
    reqs = []
    for i in range(n):
        w, h = BATCH_RESOLUTIONS[rng.integers(len(BATCH_RESOLUTIONS))]
        reqs.append(RequestSpec(i, w, h, int(rng.integers(1, 65)), frame=i))
    return scenes, reqs


def batch_small(seed: int = S.BASE_SEED, n: int = 256, tri_range=(1e3, 2e6)):
    """The scenes of batch_mix (same seed: the same scenes), one small request each: resolution
    from {64^2, 128^2, 256^2, 512^2}, spp from {1, 2, 4}."""
    scenes, _ = batch_mix(seed, n, tri_range)
    rng = np.random.default_rng(seed ^ 0x5A11)
    reqs = []
    for i in range(n):
        w, h = SMALL_RESOLUTIONS[rng.integers(len(SMALL_RESOLUTIONS))]
        reqs.append(RequestSpec(i, w, h, int(SMALL_SPP[rng.integers(len(SMALL_SPP))]), frame=i))
    return scenes, reqs


def served_small(seed: int = S.BASE_SEED, n_scenes: int = 32, n_requests: int = 512,
                 rate: float = 2000.0, tri_range=(1e4, 5e6)):
    """The resident scenes of served_stream and n_requests Poisson arrivals at `rate` per second
    of small requests: resolution from {64^2, 128^2, 256^2, 512^2}, spp from {1, 2, 4}."""
    scenes, _ = served_stream(seed, n_scenes, 0, rate, tri_range)
    rng = np.random.default_rng(seed ^ 0x5E11)
    t = 0.0
    reqs = []
    for i in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        w, h = SMALL_RESOLUTIONS[rng.integers(len(SMALL_RESOLUTIONS))]
        spp = int(SMALL_SPP[rng.integers(len(SMALL_SPP))])
        reqs.append(RequestSpec(int(rng.integers(n_scenes)), w, h, spp, frame=i, arrival_s=t))
    return scenes, reqs


def served_stream(seed: int = S.BASE_SEED, n_scenes: int = 32, n_requests: int = 96,
                  rate: float = 200.0, tri_range=(1e4, 5e6), upload_fraction: float = 0.05):
    """n_scenes resident scenes (triangles log-uniform in tri_range) and n_requests Poisson
    arrivals at `rate` per second; resolution from {512^2, 1024^2, 1920x1080}, spp from
    {1, 4, 16, 64}; a fraction of the requests brings a new 100k-triangle soup."""
    rng = np.random.default_rng(seed)
    scenes = [scene_spec(rng, *tri_range) for _ in range(n_scenes)]
    t = 0.0
    reqs = []
    for i in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        w, h = SERVED_RESOLUTIONS[rng.integers(len(SERVED_RESOLUTIONS))]
        spp = SERVED_SPP[rng.integers(len(SERVED_SPP))]
        up = None
        if rng.uniform() < upload_fraction:
            up = SceneSpec("soup", 100_000, int(rng.integers(1 << 62)))
        reqs.append(RequestSpec(int(rng.integers(n_scenes)), w, h, spp, frame=i, arrival_s=t,
                                upload=up))
    return scenes, reqs


def upload_all(ctx: S.Context, specs, threads: int = 16):
    """Builds and uploads the scenes on a thread pool (generation and BVH construction run in
    the library without the GIL); returns the scene ids in order."""
    def one(spec):
        return ctx.upload(spec.build())
    with ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, specs))


def _rotation(rng: np.random.Generator) -> np.ndarray:
    """A uniformly distributed rotation (unit quaternion from a normal 4-vector)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def instanced_scene(seed: int = S.BASE_SEED, n_meshes: int = 50, n_u: int = 250, n_v: int = 101,
                    n_instances: int = 1000, n_textures: int = 256, tex_size: int = 512,
                    bands: int = 6, box: float = 100.0, env_size=(1024, 512)) -> S.SceneData:
    """The instanced configuration: n_meshes bumpy closed meshes of 2 n_u (n_v - 1) triangles
    (50 x 50,000 by default), each split into `bands` latitude bands with their own material and
    albedo texture (n_textures sRGB value-noise RGBA8 textures, tex_size^2), placed by n_instances
    instances under random affine transforms (uniform rotation, scale in [0.5, 2], translation in
    a box^3 cube), lit by a Gaussian-lobe environment. Materials: 60 % Lambert, 40 % the OpenPBR
    GGX/Lambert Fresnel mix with roughness in [0.1, 0.6]."""
    rng = np.random.default_rng(seed)
    textures = [(S.noise_texture(seed * 7919 + 17 + t, tex_size, tex_size), True)
                for t in range(n_textures)]
    verts, idx, geoms, mats, blas = [], [], [], [], []
    v_off = t_off = 0
    for m in range(n_meshes):
        v, i = S.blob(seed * 104729 + 1000 + m, n_u, n_v)
        rows = n_v - 1
        first_geom = len(geoms)
        for b in range(bands):
            r0, r1 = b * rows // bands, (b + 1) * rows // bands
            g = np.zeros(1, N.GEOMETRY_DTYPE)
            g["first_vertex"] = v_off
            g["first_triangle"] = t_off + 2 * n_u * r0
            g["triangle_count"] = 2 * n_u * (r1 - r0)
            g["material_id"] = len(mats)
            g["flags"] = 0
            g["instance_mask"] = 0xFF
            geoms.append(g)
            mat = np.zeros(1, N.MATERIAL_DTYPE)
            lambert = rng.uniform() < 0.6
            tint = rng.uniform(0.7, 1.0, size=3)
            roughness = rng.uniform(0.1, 0.6)
            mat["model"] = N.MATERIAL_DIFFUSE if lambert else N.MATERIAL_OPENPBR
            mat["base_color"] = tint
            mat["specular_alpha"] = roughness * roughness
            mat["specular_weight"] = 0.0 if lambert else 1.0
            mat["specular_ior"] = 1.5
            mat["transmission_color"] = 1.0
            mat["base_color_texture"] = (m * bands + b) % n_textures
            mats.append(mat)
        blas.append((first_geom, bands))
        verts.append(v)
        idx.append(i)
        v_off += len(v)
        t_off += len(i)
    inst = np.zeros(n_instances, N.INSTANCE_DTYPE)
    for k in range(n_instances):
        M = _rotation(rng) * rng.uniform(0.5, 2.0)
        t = rng.uniform(0.0, box, size=3)
        inst[k]["blas"] = rng.integers(n_meshes)
        inst[k]["mask"] = 0xFF
        inst[k]["object_to_world"] = np.concatenate([M, t[:, None]], axis=1).reshape(12)
    b = np.array(blas, dtype=np.uint32).view(N.BLAS_DTYPE).reshape(-1)
    env = S.env_lobes(seed ^ 0x5E, *env_size) if env_size else None
    return S.SceneData(np.concatenate(verts), np.concatenate(idx), np.concatenate(geoms),
                       np.concatenate(mats), env, blas_ranges=b, instances=inst,
                       textures=textures)


def instanced_camera(width: int, height: int, box: float = 100.0):
    c = 0.5 * box
    return S.look_at((c, c, -0.45 * box), (c, c, c), (0.0, 1.0, 0.0), 60.0, width / height)

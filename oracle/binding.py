"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg load this module; the
product path never does. ``load()`` builds ``oracle/_build/liboracle.so`` with the Makefile
beside this file when it is missing or older than its sources.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
SOURCES = [HERE / "oracle.cpp", HERE / "oracle_math.h", HERE.parent / "include" / "gbpt.h",
           HERE.parent / "merian_gb300" / "csrc" / "scenegen.cpp",
           HERE.parent / "merian_gb300" / "csrc" / "host_common.h"]

_lib = None


def build() -> Path:
    stale = not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in SOURCES)
    if stale:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        vp, u32, u64, i32, f32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
        lib.oracle_scene_create.restype = vp
        lib.oracle_scene_create.argtypes = [vp, u64, vp, u64, vp, u32, vp, u32, vp, u32, u32, vp,
                                            f32]
        lib.oracle_scene_destroy.argtypes = [vp]
        lib.oracle_trace_primary.argtypes = [vp, vp, u32, u32, u32, i32, vp, vp]
        lib.oracle_trace_rays.argtypes = [vp, vp, u32, u32, i32, i32, vp, vp, vp]
        lib.oracle_render.argtypes = [vp, vp, vp, i32, i32, vp, vp, vp, vp]
        lib.oracle_num_threads.restype = i32
        lib.oracle_gbuffer.argtypes = [vp, vp, u32, u32, u32, vp]
        lib.oracle_scene_set_instances.argtypes = [vp, vp, u32, vp, u32]
        lib.oracle_scene_set_textures.argtypes = [vp, vp, u32]
        lib.oracle_bsdf_check.argtypes = [i32, vp, vp, f32, f32, vp, f32, f32, u32, u32, vp]
        lib.oracle_material_samples.argtypes = [vp, i32, f32, vp, u32, u32, vp]
        fp = C.POINTER(C.c_float)
        lib.oracle_camera_look_at.argtypes = [fp, fp, fp, f32, f32, f32, f32, vp]
        lib.oracle_camera_look_at.restype = i32
        lib.oracle_alias_table.argtypes = [vp, u32, vp]
        # the seeded scene generators, compiled into this library from the package's source
        from merian_gb300 import _native as N
        for name, res, args in N.EXPORTS:
            if name.startswith("gbpt_gen_"):
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
        _lib = lib
    return _lib


def alias_table(w: np.ndarray) -> np.ndarray:
    """The package's alias table of weights w: (n, 2) uint32, (keep probability bits, alias)."""
    w = np.ascontiguousarray(w, np.float64)
    out = np.zeros((len(w), 2), np.uint32)
    load().oracle_alias_table(_p(w), len(w), _p(out))
    return out


def _p(a) -> int:
    return a.ctypes.data if a is not None and a.size else 0


class OracleScene:
    """The oracle's own copy of a scene (same host arrays the GPU receives)."""

    def __init__(self, scene):
        lib = load()
        self._keep = scene
        env = None if scene.env is None else np.ascontiguousarray(scene.env, np.float32)
        self._env = env
        m = np.ascontiguousarray(np.asarray(scene.env_to_local, np.float32).reshape(9))
        self._m = m
        self.h = lib.oracle_scene_create(
            _p(scene.vertices), len(scene.vertices), _p(scene.indices), scene.triangle_count,
            _p(scene.geometries), len(scene.geometries), _p(scene.materials),
            len(scene.materials), _p(env), 0 if env is None else env.shape[1],
            0 if env is None else env.shape[0], _p(m), float(scene.env_intensity))
        d, self._desc_keep = scene.desc()
        if getattr(scene, "textures", None):
            lib.oracle_scene_set_textures(self.h, C.cast(d.textures, C.c_void_p).value,
                                          d.texture_count)
        if getattr(scene, "instances", None) is not None and len(scene.instances):
            if lib.oracle_scene_set_instances(self.h, d.blas_ranges, d.blas_count, d.instances,
                                              d.instance_count) != 0:
                raise ValueError("oracle: bad instances")

    def close(self):
        if self.h:
            load().oracle_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace_primary(self, camera, width: int, height: int, mask: int = 0xFF,
                      fp64: bool = True, hit_dtype=None):
        hits = np.zeros(width * height, hit_dtype)
        t64 = np.zeros(width * height, np.float64)
        load().oracle_trace_primary(self.h, C.addressof(camera), width, height, mask, int(fp64),
                                    _p(hits), _p(t64))
        return hits, t64

    def trace_rays(self, rays: np.ndarray, mask: int = 0xFF, fp64: bool = False,
                   any_hit: bool = False, hit_dtype=None):
        hits = np.zeros(len(rays), hit_dtype)
        nn, nt = C.c_uint64(), C.c_uint64()
        load().oracle_trace_rays(self.h, _p(rays), len(rays), mask, int(fp64), int(any_hit),
                                 _p(hits), C.addressof(nn), C.addressof(nt))
        return hits, nn.value, nt.value

    def gbuffer(self, camera, width: int, height: int, mask: int = 0xFF, texel_dtype=None):
        """FP32 GBuffer texels (gbpt_gbuffer_texel layout), row-major."""
        out = np.zeros(width * height, texel_dtype)
        load().oracle_gbuffer(self.h, C.addressof(camera), width, height, mask, _p(out))
        return out

    def render(self, camera, params, fp64: bool = True, threads: int = 0, lum4: bool = False):
        """(rgba (n,4) float64, mean of squared per-sample rgb (n,3), traced rays); with lum4 a
        fourth element, the per-pixel mean of luminance^4 (n,): the second moment of the samples
        the `a` channel (mean luminance^2) averages."""
        n = params.pixel_count or params.width * params.height
        rgba = np.zeros((n, 4), np.float64)
        sq = np.zeros((n, 3), np.float64)
        l4 = np.zeros(n, np.float64) if lum4 else None
        rays = C.c_uint64()
        load().oracle_render(self.h, C.addressof(camera), C.addressof(params), int(fp64), threads,
                             _p(rgba), _p(sq), _p(l4) if lum4 else None, C.addressof(rays))
        if lum4:
            return rgba, sq, rays.value, l4
        return rgba, sq, rays.value


def generator() -> C.CDLL:
    """This library as the source of the seeded scene generators (gbpt_gen_*): pass it as
    ``lib=`` to ``merian_gb300.scene``'s factories to build a scene without the CUDA library."""
    return load()


def look_at(position, target, up=(0.0, 1.0, 0.0), vfov_deg: float = 40.0, aspect: float = 1.0,
            near: float = 0.1, far: float = 1000.0):
    """merian's pinhole basis from the oracle's own restatement (oracle_camera_look_at)."""
    import math
    from merian_gb300 import _native as N
    cam = N.Camera()
    f3 = C.c_float * 3
    rc = load().oracle_camera_look_at(f3(*position), f3(*target), f3(*up), math.radians(vfov_deg),
                                      aspect, near, far, C.addressof(cam))
    if rc != 0:
        raise ValueError("oracle_camera_look_at: bad arguments")
    return cam


def workload_camera(name: str, width: int | None = None, height: int | None = None):
    """The camera of a named workload (merian_gb300.scene.WORKLOADS), from look_at above."""
    from merian_gb300 import scene as S
    w = S.WORKLOADS[name]
    c = w["camera"]
    return look_at(c["position"], c["target"], (0.0, 1.0, 0.0), c["vfov_deg"],
                   (width or w["width"]) / (height or w["height"]))


def cwbvh_trace(nodes: np.ndarray, tris: np.ndarray, rays: np.ndarray, mask: int = 0xFF,
                any_hit: bool = False, hit_dtype=None):
    """Hits of rays through a single-level CWBVH of gbpt_bvh_build (nodes (n, 80) uint8, triangle
    records (m, 48) uint8), and per ray (nodes visited, triangles tested): a host walk in the
    device's traversal order with its box decisions (oracle_cwbvh_trace)."""
    lib = load()
    lib.oracle_cwbvh_trace.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                       C.c_void_p, C.c_uint32, C.c_uint32, C.c_int, C.c_void_p,
                                       C.c_void_p]
    nodes = np.ascontiguousarray(nodes, np.uint8)
    tris = np.ascontiguousarray(tris, np.uint8)
    rays = np.ascontiguousarray(rays)
    hits = np.zeros(len(rays), hit_dtype)
    counts = np.zeros((len(rays), 2), np.uint32)
    rc = lib.oracle_cwbvh_trace(_p(nodes), len(nodes), _p(tris), len(tris), _p(rays), len(rays),
                                mask, int(any_hit), _p(hits), _p(counts))
    if rc != 0:
        raise ValueError("oracle_cwbvh_trace: bad arguments")
    return hits, counts


def bounce_rays(osc: "OracleScene", camera, params, ray_dtype, cap: int = 1 << 24):
    """The closest-hit bounce rays the FP32 oracle traces for params' pixels (oracle_bounce_rays):
    a sample of the workload's bounce-ray distribution, as a ray_dtype array."""
    lib = load()
    lib.oracle_bounce_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_uint64, C.c_void_p]
    out = np.zeros(cap, ray_dtype)
    n = C.c_uint64()
    lib.oracle_bounce_rays(osc.h, C.addressof(camera), C.addressof(params), _p(out), cap,
                           C.addressof(n))
    return out[:min(n.value, cap)]


def num_threads() -> int:
    return load().oracle_num_threads()


BSDF_KINDS = {"lambert": 0, "ggx": 1, "conductor": 2, "rough_dielectric": 3, "fresnel_mix": 4}


def bsdf_check(kind: str, wi, albedo=(0.8, 0.5, 0.2), alpha: float = 0.3,
               alpha_y: float | None = None, f0=(0.95, 0.64, 0.54), ior_f0: float = 0.04,
               eta: float = 1.0 / 1.5, n_samples: int = 1 << 18, seed: int = 0x1234567) -> dict:
    """The reference's BSDF property checks (tests/bsdf/bsdf-checks.slang) on the oracle BSDFs."""
    out = np.zeros(16, np.float32)
    wi = np.asarray(wi, np.float32)
    al = np.asarray(albedo, np.float32)
    f0a = np.asarray(f0, np.float32)
    load().oracle_bsdf_check(BSDF_KINDS[kind], _p(wi), _p(al), alpha,
                             alpha if alpha_y is None else alpha_y, _p(f0a), ior_f0, eta,
                             n_samples, seed, _p(out))
    return unpack_check(out, n_samples)


def material_samples(material: np.ndarray, front: bool, ior: float, wi, seed: int, n: int):
    """(n, 12) float32: wo, pdf, weight, valid, eval(wi, wo), pdf(wi, wo) per sample."""
    out = np.zeros((n, 12), np.float32)
    m = np.ascontiguousarray(material)
    w = np.asarray(wi, np.float32)
    load().oracle_material_samples(_p(m), int(front), ior, _p(w), seed, n, _p(out))
    return out


def bsdf_integrals(kind: str, wi, alpha: float = 0.3, eta: float = 1 / 1.5,
                   ior_f0: float = 0.04, n_samples: int = 1 << 20, n_theta: int = 1024) -> dict:
    """Sampler vs evaluation: furnace and valid fraction against the full-sphere quadrature of
    eval and pdf (FP64)."""
    out = np.zeros(4, np.float64)
    w = np.asarray(wi, np.float64)
    lib = load()
    lib.oracle_bsdf_integrals.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_double,
                                          C.c_double, C.c_uint32, C.c_uint32, C.c_void_p]
    lib.oracle_bsdf_integrals(BSDF_KINDS[kind], _p(w), alpha, eta, ior_f0, n_samples, n_theta,
                              _p(out))
    return dict(furnace=out[0], eval_integral=out[1], valid=out[2], pdf_integral=out[3])


def unpack_check(out: np.ndarray, n_samples: int) -> dict:
    return dict(furnace=out[0:3].astype(np.float64), furnace_stderr=out[3:6].astype(np.float64),
                mean_cos=float(out[6]), stderr_cos=float(out[7]), valid=int(out[8]),
                max_weight_err=float(out[9]), max_pdf_err=float(out[10]),
                pdf_integral=float(out[11]), max_recip_err=float(out[12]), n=n_samples)


def primary_points(osc: "OracleScene", camera, params) -> np.ndarray:
    """FP32 primary shading points, 24 floats per pixel (gbpt_debug_primary_points layout)."""
    n = params.pixel_count or params.width * params.height
    out = np.zeros((n, 24), np.float32)
    lib = load()
    lib.oracle_primary_points.argtypes = [C.c_void_p] * 4
    lib.oracle_primary_points(osc.h, C.addressof(camera), C.addressof(params), _p(out))
    return out

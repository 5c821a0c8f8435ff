"""ctypes binding of the C ABI in ``include/gbpt.h`` (``merian_gb300/libgbpt.so``).

The struct layouts below mirror the header one to one; numpy structured dtypes are provided for
the array types so scenes can be built and passed without copies.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libgbpt.so"

GBPT_OK = 0
GBPT_ERR_INVALID = -1
GBPT_ERR_CUDA = -2
GBPT_ERR_NO_MEMORY = -3
GBPT_ERR_NOT_FOUND = -4
GBPT_ERR_DEVICE = -5
GBPT_ERR_BUSY = -6
GBPT_ERR_CANCELLED = -7

MESH_FLIP_FACING = 0x8
MESH_TWO_SIDED = 0x10
MESH_HAS_TANGENTS = 0x20
MESH_FLAT_SHADING = 0x40
MESH_USE_ENV_MAP = 0x80
MESH_ALPHA_TEST = 0x100

MATERIAL_DIFFUSE = 0
MATERIAL_OPENPBR = 1
MATERIAL_OPENPBR_TRANSMISSION = 2

VERTEX_DTYPE = np.dtype([("position", "<f4", 3), ("encoded_normal", "<u4"), ("uv", "<u4"),
                         ("encoded_tangent", "<u4")])
GEOMETRY_DTYPE = np.dtype([("first_vertex", "<u4"), ("first_triangle", "<u4"),
                           ("triangle_count", "<u4"), ("material_id", "<u4"), ("flags", "<u4"),
                           ("instance_mask", "<u4")])
MATERIAL_DTYPE = np.dtype([("model", "<u4"), ("base_color", "<f4", 3), ("metalness", "<f4"),
                           ("specular_alpha", "<f4", 2), ("specular_weight", "<f4"),
                           ("specular_ior", "<f4"), ("emission", "<f4", 3),
                           ("transmission_weight", "<f4"), ("transmission_color", "<f4", 3),
                           ("base_color_texture", "<i4"), ("alpha_texture", "<i4"),
                           ("reserved", "<u4", 2)])
HIT_DTYPE = np.dtype([("instance_id", "<u4"), ("instance_index", "<u4"), ("primitive_id", "<u4"),
                      ("geometry_index", "<u4"), ("barycentrics", "<f4", 2), ("t", "<f4"),
                      ("reserved", "<u4")])
RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("tmin", "<f4"), ("direction", "<f4", 3),
                      ("tmax", "<f4")])
INSTANCE_DTYPE = np.dtype([("blas", "<u4"), ("mask", "<u4"), ("object_to_world", "<f4", 12)])
BLAS_DTYPE = np.dtype([("first_geometry", "<u4"), ("geometry_count", "<u4")])
assert INSTANCE_DTYPE.itemsize == 56
GBUFFER_DTYPE = np.dtype([("encoded_normal", "<u4"), ("grad_z", "<u4"), ("instance_id", "<u4"),
                          ("primitive_id", "<u4"), ("geometry_index", "<u2"),
                          ("instance_index", "<u2"), ("barycentrics", "<u4"),
                          ("motion", "<f4", 2), ("linear_z", "<f4"), ("delta_z", "<f4"),
                          ("albedo", "<f4", 3), ("emission", "<f4", 3)])
assert GBUFFER_DTYPE.itemsize == 64
assert VERTEX_DTYPE.itemsize == 24 and GEOMETRY_DTYPE.itemsize == 24
assert MATERIAL_DTYPE.itemsize == 80 and HIT_DTYPE.itemsize == 32 and RAY_DTYPE.itemsize == 32


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("U", C.c_float * 3), ("V", C.c_float * 3),
                ("W", C.c_float * 3), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("jitter", C.c_float * 2)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_int32),
                ("max_path_length", C.c_int32), ("emission_on_primary", C.c_int32),
                ("instance_mask", C.c_uint32), ("demodulate_albedo", C.c_int32),
                ("sort_materials", C.c_int32), ("frame", C.c_uint32), ("nee", C.c_int32),
                ("rr_depth", C.c_int32), ("pixels", C.POINTER(C.c_uint32)),
                ("pixel_count", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("device_ms", C.c_double),
                ("trace_ms", C.c_double), ("shade_ms", C.c_double), ("shadow_ms", C.c_double),
                ("other_ms", C.c_double), ("trace_launches", C.c_uint64),
                ("trace_rays", C.c_uint64), ("nodes_visited", C.c_uint64),
                ("tris_tested", C.c_uint64), ("node_steps", C.c_uint64),
                ("node_lanes", C.c_uint64), ("tri_steps", C.c_uint64),
                ("tri_lanes", C.c_uint64)]


class EnvMap(C.Structure):
    _fields_ = [("texels", C.POINTER(C.c_float)), ("width", C.c_uint32), ("height", C.c_uint32),
                ("to_local", C.c_float * 9), ("intensity", C.c_float)]


class Texture(C.Structure):
    _fields_ = [("texels", C.POINTER(C.c_uint8)), ("width", C.c_uint32), ("height", C.c_uint32),
                ("srgb", C.c_uint32), ("reserved", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("vertex_count", C.c_uint64),
                ("indices", C.c_void_p), ("triangle_count", C.c_uint64),
                ("geometries", C.c_void_p), ("geometry_count", C.c_uint32),
                ("materials", C.c_void_p), ("material_count", C.c_uint32),
                ("env", C.POINTER(EnvMap)), ("textures", C.POINTER(Texture)),
                ("texture_count", C.c_uint32), ("blas_ranges", C.c_void_p),
                ("blas_count", C.c_uint32), ("instances", C.c_void_p),
                ("instance_count", C.c_uint32)]


class LoadedInfo(C.Structure):
    _fields_ = [("desc", SceneDesc), ("camera", Camera), ("width", C.c_uint32),
                ("height", C.c_uint32), ("warning_count", C.c_uint32), ("reserved", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("reserved", C.c_uint32), ("camera", Camera),
                ("params", RenderParams), ("out_host", C.c_void_p), ("out_device", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("wave_paths", C.c_uint64), ("arena_bytes", C.c_uint64),
                ("use_graphs", C.c_int32), ("max_active", C.c_uint32)]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("error", C.c_int32), ("submit_s", C.c_double),
                ("admit_s", C.c_double), ("done_s", C.c_double), ("samples", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("queued", C.c_uint64), ("active", C.c_uint64), ("completed", C.c_uint64),
                ("ticks", C.c_uint64), ("kernel_launches", C.c_uint64), ("paths", C.c_uint64),
                ("arena_bytes", C.c_uint64), ("wave_paths", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("wave_paths", C.c_uint64), ("sort_materials", C.c_int32),
                ("use_graphs", C.c_int32), ("bvh_build", C.c_int32), ("streams", C.c_int32),
                ("trace_refill_lanes", C.c_int32), ("trace_postpone_lanes", C.c_int32),
                ("trace_blocks_per_sm", C.c_int32)]


AUTOTUNE_CANDIDATES = 32


BVH_SPLIT, BVH_FAST, BVH_MEDIUM = 0, 1, 2


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)

# (name, restype, argtypes) of every exported entry point declared in include/gbpt.h
EXPORTS = [
    ("gbpt_render_batch", C.c_int, [C.c_void_p, C.POINTER(Request), C.c_uint32,
                                    C.POINTER(RenderStats)]),
    ("gbpt_set_graphs", C.c_int, [C.c_void_p, C.c_int]),
    ("gbpt_set_tuning", C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    ("gbpt_get_tuning", C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    ("gbpt_autotune", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.POINTER(RenderParams),
                                C.POINTER(Tuning), C.POINTER(C.c_double)]),
    ("gbpt_clock", C.c_double, []),
    ("gbpt_server_start", C.c_int, [C.c_void_p, C.POINTER(ServerConfig)]),
    ("gbpt_server_stop", C.c_int, [C.c_void_p]),
    ("gbpt_server_submit", C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    ("gbpt_server_poll", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(RequestStatus)]),
    ("gbpt_server_wait", C.c_int, [C.c_void_p, C.c_uint64, C.c_double,
                                   C.POINTER(RequestStatus)]),
    ("gbpt_server_cancel", C.c_int, [C.c_void_p, C.c_uint64]),
    ("gbpt_server_release", C.c_int, [C.c_void_p, C.c_uint64]),
    ("gbpt_server_info", C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    ("gbpt_gbuffer", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.c_uint32, C.c_uint32,
                               C.c_uint32, C.c_void_p]),
    ("gbpt_accumulate", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                  C.c_float, C.c_float, C.c_int]),
    ("gbpt_error_metrics", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                     C.POINTER(C.c_double)]),
    ("gbpt_image_write_pfm", C.c_int, [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                       C.c_uint32]),
    ("gbpt_image_read_pfm", C.c_int, [C.c_char_p, C.c_void_p, C.c_uint32,
                                      C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("gbpt_abi_version", C.c_uint32, []),
    ("gbpt_last_error", C.c_char_p, []),
    ("gbpt_create", C.c_int, [C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]),
    ("gbpt_destroy", C.c_int, [C.c_void_p]),
    ("gbpt_synchronize", C.c_int, [C.c_void_p]),
    ("gbpt_memory_info", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint64)]),
    ("gbpt_set_profiling", C.c_int, [C.c_void_p, C.c_int]),
    ("gbpt_scene_create", C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_uint32)]),
    ("gbpt_scene_destroy", C.c_int, [C.c_void_p, C.c_uint32]),
    ("gbpt_scene_stats", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint32)]),
    ("gbpt_render", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.POINTER(RenderParams),
                              C.c_void_p, C.POINTER(RenderStats)]),
    ("gbpt_render_device", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera),
                                     C.POINTER(RenderParams), C.c_void_p,
                                     C.POINTER(RenderStats)]),
    ("gbpt_render_device_noalloc", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera),
                                             C.POINTER(RenderParams), C.c_void_p]),
    ("gbpt_trace_primary", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.c_uint32,
                                     C.c_uint32, C.c_uint32, C.c_void_p]),
    ("gbpt_trace", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int,
                             C.c_void_p]),
    ("gbpt_trace_counted", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32,
                                     C.c_int, C.c_void_p, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]),
    ("gbpt_debug_material_samples", C.c_int, [C.c_void_p, C.c_int, C.c_float,
                                              C.POINTER(C.c_float), C.c_uint32, C.c_uint32,
                                              C.c_void_p]),
    ("gbpt_debug_bsdf_check", C.c_int, [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                        C.c_float, C.c_float, C.POINTER(C.c_float), C.c_float,
                                        C.c_float, C.c_uint32, C.c_uint32, C.c_void_p]),
    ("gbpt_debug_primary_points", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera),
                                            C.POINTER(RenderParams), C.c_void_p]),
    ("gbpt_camera_look_at", C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float),
                                      C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float,
                                      C.c_float, C.POINTER(Camera)]),
    ("gbpt_encode_normal", C.c_uint32, [C.POINTER(C.c_float)]),
    ("gbpt_pack_half2", C.c_uint32, [C.c_float, C.c_float]),
    ("gbpt_gen_cornell", C.c_int, [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("gbpt_gen_cornell_tess", C.c_int, [C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
    ("gbpt_gen_soup", C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p]),
    ("gbpt_gen_blob", C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("gbpt_gen_noise_texture", C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p]),
    ("gbpt_load_pbrt", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    ("gbpt_load_gltf", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    ("gbpt_image_read_png", C.c_int, [C.c_char_p, C.c_void_p, C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]),
    ("gbpt_loaded_scene_info", C.c_int, [C.c_void_p, C.POINTER(LoadedInfo)]),
    ("gbpt_loaded_scene_warning", C.c_char_p, [C.c_void_p, C.c_uint32]),
    ("gbpt_loaded_scene_free", None, [C.c_void_p]),
    ("gbpt_gen_env", C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p]),
    ("gbpt_bvh_build", C.c_int, [C.POINTER(SceneDesc), C.c_int32, C.POINTER(C.c_void_p)]),
    ("gbpt_bvh_info", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                C.POINTER(C.c_uint32)]),
    ("gbpt_bvh_free", None, [C.c_void_p]),
    ("gbpt_graph_create", C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    ("gbpt_graph_destroy", C.c_int, [C.c_void_p]),
    ("gbpt_graph_node_count", C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    ("gbpt_graph_node", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_char_p),
                                  C.POINTER(C.c_char_p)]),
    ("gbpt_graph_warning_count", C.c_uint32, [C.c_void_p]),
    ("gbpt_graph_warning", C.c_char_p, [C.c_void_p, C.c_uint32]),
    ("gbpt_graph_set_property", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                          C.POINTER(C.c_uint32)]),
    ("gbpt_graph_get_property", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                          C.c_uint64, C.POINTER(C.c_uint64)]),
    ("gbpt_graph_run", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.c_uint32,
                                 C.c_uint32, C.c_uint32]),
    ("gbpt_debug_fail_allocations", C.c_int, [C.c_int64, C.c_int64]),
    ("gbpt_graph_option", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_char_p),
                                    C.POINTER(C.c_char_p)]),
    ("gbpt_graph_set_option", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p,
                                        C.POINTER(C.c_uint32)]),
    ("gbpt_graph_to_json", C.c_int, [C.c_void_p, C.c_char_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("gbpt_graph_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("gbpt_graph_load", C.c_int, [C.c_void_p, C.c_char_p]),
    ("gbpt_graph_output", C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_uint64,
                                    C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                    C.POINTER(C.c_uint32)]),
]

_lib = None


class GbptError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"gbpt error {code}: {message}")
        self.code = code


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads libgbpt.so. Raises if it has not been built: there is no fallback implementation."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    # GBPT_LIBRARY selects another build of the library (a tuning variant)
    p = Path(path) if path else Path(os.environ.get("GBPT_LIBRARY", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m merian_gb300.build` "
                           "(the path tracer has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, res, args in EXPORTS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != GBPT_OK:
        msg = load().gbpt_last_error()
        raise GbptError(rc, msg.decode() if msg else "")


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None and a.size else 0

/*
 * gbpt.h — C ABI of the GB300-native wavefront path tracer that stands in for merian's
 * "Render (Path-traced)" node (RenderPT).
 *
 * The reference node (src/merian-graph/nodes/render_pt/render_pt.cpp:94-124) binds a Vulkan
 * scene and launches one ray-generation thread per pixel (render_pt.slang:92-130). Here the
 * same per-sample loop runs as CUDA wavefront kernels for sm_103a; this header is the only
 * boundary a host (the C++ node shim, a merian plugin, ctypes) needs. Conventions:
 *   - plain C structs and pointers, no C++ or CUDA types;
 *   - every call returns an int status (GBPT_OK = 0, negative on error) and the message of the
 *     last failing call on this thread is available from gbpt_last_error();
 *   - the caller owns host buffers, the library owns device memory and frees it in
 *     gbpt_scene_destroy()/gbpt_destroy();
 *   - one context drives one CUDA device and one stream; calls on one context are serialised
 *     by an internal mutex.
 */
#ifndef GBPT_H
#define GBPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define GBPT_API __declspec(dllexport)
#else
#define GBPT_API __attribute__((visibility("default")))
#endif

#define GBPT_ABI_VERSION 1u

/* ---- status codes ------------------------------------------------------------------------ */
#define GBPT_OK 0
#define GBPT_ERR_INVALID (-1)   /* bad argument (null pointer, size out of range, bad id) */
#define GBPT_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define GBPT_ERR_NO_MEMORY (-3) /* device or host allocation failed, or admission refused */
#define GBPT_ERR_NOT_FOUND (-4) /* unknown scene / request id */
#define GBPT_ERR_DEVICE (-5)    /* a kernel raised its error flag (stack overflow, bad index) */
#define GBPT_ERR_BUSY (-6)      /* request not finished yet (gbpt_server_poll) */
#define GBPT_ERR_CANCELLED (-7) /* request was cancelled before it finished */

/* ---- mesh flags: identical bit values to merian::Scene::MeshFlags (scene.hpp:39-58) -------- */
#define GBPT_MESH_FLIP_FACING 0x8u   /* front winding is clockwise: face normal negated */
#define GBPT_MESH_TWO_SIDED 0x10u    /* no back-face culling; back hits flip the frame */
#define GBPT_MESH_HAS_TANGENTS 0x20u /* per-vertex tangents are meaningful */
#define GBPT_MESH_FLAT_SHADING 0x40u /* shading normal = face normal */
#define GBPT_MESH_USE_ENV_MAP 0x80u  /* hits shade as the environment along the ray */

/* ---- material models (merian MaterialSystem type ids, material-system.slang:51-56) --------- */
#define GBPT_MATERIAL_DIFFUSE 0u              /* DiffuseMaterial (diffuse-material.slang) */
#define GBPT_MATERIAL_OPENPBR 1u              /* OpenPBRMaterial<> (openpbr-material.slang) */
#define GBPT_MATERIAL_OPENPBR_TRANSMISSION 2u /* OpenPBRMaterial<TRANSMISSION=true> */

/* Vertex layout of merian's PackedVertexData (scene-data.slangh:75-101), 24 bytes. */
typedef struct gbpt_packed_vertex {
    float position[3];
    uint32_t encoded_normal;  /* oct-encoded, packSnorm2x16 (encoding.slang:6-30) */
    uint32_t uv;              /* half2: x in the low 16 bits */
    uint32_t encoded_tangent; /* oct direction in the upper 31 bits, LSB = handedness < 0 */
} gbpt_packed_vertex;

/* One geometry (merian GeometryData, scene-data.slangh:119-129): a triangle range sharing one
 * material and one set of mesh flags. Indices are relative to first_vertex. */
typedef struct gbpt_geometry {
    uint32_t first_vertex;
    uint32_t first_triangle; /* into gbpt_scene_desc.indices, in triangles */
    uint32_t triangle_count;
    uint32_t material_id;
    uint32_t flags; /* GBPT_MESH_* */
    uint32_t instance_mask; /* 8-bit cull mask of the TLAS instance holding this geometry */
} gbpt_geometry;

/* Material record, 80 bytes. DIFFUSE reads base_color (and base_color_texture); the OpenPBR
 * models read the rest with the reference's field meaning (openpbr-material.slang:173-190).
 * specular_alpha is GGX alpha (roughness squared), clamped at sample time to
 * 0.0316^2 (material.slang:23). */
typedef struct gbpt_material {
    uint32_t model; /* GBPT_MATERIAL_* */
    float base_color[3];
    float metalness;
    float specular_alpha[2];
    float specular_weight;
    float specular_ior;
    float emission[3];
    float transmission_weight;
    float transmission_color[3];
    int32_t base_color_texture; /* -1 = none */
    uint32_t reserved[3];
} gbpt_material;

/* RGBA8 texture (sRGB is not applied: values are linear / 255). */
typedef struct gbpt_texture {
    const uint8_t* texels; /* width*height*4 bytes, row-major */
    uint32_t width;
    uint32_t height;
} gbpt_texture;

/* Lat-long environment (merian LatLongMap, environment-map.slang:23-35): RGBA32F texels,
 * bilinear filtering with repeat addressing, level 0; to_local is a row-major 3x3 rotation. */
typedef struct gbpt_env_map {
    const float* texels; /* width*height*4 floats, row-major, row 0 = v in [0, 1/height) */
    uint32_t width;
    uint32_t height;
    float to_local[9];
    float intensity;
} gbpt_env_map;

/* A TLAS instance (two-level scenes): geometries [first_geometry, first_geometry+count) are one
 * BLAS, placed by a row-major 3x4 object-to-world affine transform. */
typedef struct gbpt_instance {
    uint32_t blas; /* index into gbpt_scene_desc.blas_ranges */
    uint32_t mask;
    float object_to_world[12];
} gbpt_instance;

typedef struct gbpt_blas_range {
    uint32_t first_geometry;
    uint32_t geometry_count;
} gbpt_blas_range;

typedef struct gbpt_scene_desc {
    const gbpt_packed_vertex* vertices;
    uint64_t vertex_count;
    const uint32_t* indices; /* 3 per triangle */
    uint64_t triangle_count;
    const gbpt_geometry* geometries;
    uint32_t geometry_count;
    const gbpt_material* materials;
    uint32_t material_count;
    const gbpt_env_map* env; /* NULL: black environment (merian EmptyEnv) */
    const gbpt_texture* textures;
    uint32_t texture_count;
    /* two-level scenes; instance_count == 0 means one identity instance over all geometries */
    const gbpt_blas_range* blas_ranges;
    uint32_t blas_count;
    const gbpt_instance* instances;
    uint32_t instance_count;
} gbpt_scene_desc;

/* Pinhole camera basis exactly as merian's Camera::write_to uploads it (camera.cpp:349-367) and
 * Camera::generate_ray_pinhole reads it (camera.slang:29-56). */
typedef struct gbpt_camera {
    float position[3];
    float U[3];
    float V[3];
    float W[3];
    float near_plane;
    float far_plane;
    float jitter[2];
} gbpt_camera;

/* Per-frame parameters: the RenderPT properties (render_pt.cpp:147-186) plus the RNG lane. */
typedef struct gbpt_render_params {
    uint32_t width;
    uint32_t height;
    int32_t spp;                 /* "samples per pixel" */
    int32_t max_path_length;     /* "max path length" (segments, including the primary hit) */
    int32_t emission_on_primary; /* "emission on primary" */
    uint32_t instance_mask;      /* bits "0".."7" */
    int32_t demodulate_albedo;   /* "demodulate albedo" */
    int32_t sort_materials;      /* "shader execution reordering": material-sorted shading */
    uint32_t frame;              /* RNG lane 3, merian's scene.frame ("seed") */
    int32_t nee;                 /* next-event estimation with MIS (0 = BSDF-only estimator) */
    int32_t rr_depth;            /* Russian roulette from this path length (0 = off) */
    const uint32_t* pixels;      /* optional subset of linear pixel ids y*width+x (host) */
    uint32_t pixel_count;        /* 0 = every pixel */
} gbpt_render_params;

/* Work counters of one render call. */
typedef struct gbpt_render_stats {
    uint64_t samples;      /* pixel x spp paths */
    uint64_t rays;         /* every traced segment: camera, bounce and shadow rays */
    uint64_t shadow_rays;
    uint64_t kernel_launches;
    double device_ms;      /* device time of the call, CUDA events on the context stream */
    /* filled when profiling is enabled (gbpt_set_profiling) */
    double trace_ms;       /* closest-hit traversal launches of the bounce loop */
    double shade_ms;       /* shading / scatter launches */
    double shadow_ms;      /* NEE occlusion launches */
    double other_ms;       /* primary hits and finalisation */
    uint64_t trace_launches;
    uint64_t trace_rays;   /* rays through the closest-hit traversal launches */
    uint64_t nodes_visited; /* level 2: CWBVH nodes visited by those rays */
    uint64_t tris_tested;   /* level 2: triangles tested by those rays */
} gbpt_render_stats;

/* Closest hit of one ray, merian Hit (hit.slang:25-65) plus the distance. Misses have
 * instance_id = geometry_index = primitive_id = 0xFFFFFFFF. */
typedef struct gbpt_hit {
    uint32_t instance_id;    /* custom index: first geometry id of the instance's BLAS */
    uint32_t instance_index; /* TLAS instance */
    uint32_t primitive_id;   /* triangle within the geometry */
    uint32_t geometry_index; /* geometry within the BLAS */
    float barycentrics[2];
    float t;
    uint32_t reserved;
} gbpt_hit;

/* A ray in device memory: origin, tmin, direction, tmax (two float4). */
typedef struct gbpt_ray {
    float origin[3];
    float tmin;
    float direction[3];
    float tmax;
} gbpt_ray;

typedef struct gbpt_ctx gbpt_ctx;

/* ---- context ----------------------------------------------------------------------------- */
GBPT_API uint32_t gbpt_abi_version(void);
GBPT_API const char* gbpt_last_error(void);
/* stream: a cudaStream_t cast to an integer; 0 creates a private non-blocking stream. */
GBPT_API int gbpt_create(int device, uint64_t stream, gbpt_ctx** out_ctx);
GBPT_API int gbpt_destroy(gbpt_ctx* ctx);
GBPT_API int gbpt_synchronize(gbpt_ctx* ctx);
GBPT_API int gbpt_memory_info(gbpt_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes,
                              uint64_t* ctx_bytes);
/* Kernel profiling of later render calls with stats: 0 off, 1 per-kernel-class device times (CUDA
 * events around each launch), 2 also counts CWBVH nodes and triangles visited (instrumented
 * traversal; slower, for the bytes-per-ray roofline only). Replaces merian's Profiler scopes
 * (include/merian/vk/utils/profiler.hpp). */
GBPT_API int gbpt_set_profiling(gbpt_ctx* ctx, int level);

/* ---- scenes -------------------------------------------------------------------------------
 * Replaces merian's Scene upload + driver BLAS/TLAS build (scene.cpp:1117-1120,1836-1882): the
 * geometry is copied to HBM and a compressed 8-wide BVH (80-byte nodes) is built on the host. */
GBPT_API int gbpt_scene_create(gbpt_ctx* ctx, const gbpt_scene_desc* desc, uint32_t* out_scene);
GBPT_API int gbpt_scene_destroy(gbpt_ctx* ctx, uint32_t scene);
/* BVH statistics: nodes, triangles referenced, device bytes, maximum depth. */
GBPT_API int gbpt_scene_stats(gbpt_ctx* ctx, uint32_t scene, uint64_t* nodes, uint64_t* tris,
                              uint64_t* bytes, uint32_t* depth);

/* ---- the drop-in: RenderPT::process ---------------------------------------------------------
 * Renders params->width x height (or the listed pixels) into RGBA32F: rgb = mean radiance over
 * spp, a = mean squared YUV luminance; NaN/Inf samples are dropped but counted (render_pt.slang
 * :110-129). gbpt_render writes to a HOST buffer (copies inside the call); gbpt_render_device
 * writes to DEVICE memory, enqueued on the context stream, and returns without synchronising
 * unless stats is non-NULL. With a pixel subset the output holds pixel_count texels in list
 * order. */
GBPT_API int gbpt_render(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                         const gbpt_render_params* params, float* out_rgba_host,
                         gbpt_render_stats* stats);
GBPT_API int gbpt_render_device(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                const gbpt_render_params* params, float* out_rgba_device,
                                gbpt_render_stats* stats);

/* Rendering for callers that cannot allocate device memory while they render: a host whose own
 * allocator owns the GPU's memory, a real-time loop that must not block in cudaMalloc/cudaFree
 * (either can synchronise the whole device), or a process whose memory budget is fixed when it
 * starts. It runs the same wavefront as gbpt_render_device, but every scratch buffer comes from a
 * fixed 64 MiB device array compiled into the library, held by each GPU that loads the library
 * until the process exits; this call allocates nothing. The scene must already be resident
 * (gbpt_scene_create, an earlier set-up step) and out_rgba_device is caller-owned device memory.
 * Limits: spp at most the paths one pass over the array holds (242,182), a pixel
 * subset of at most 65,536 entries; larger requests return GBPT_ERR_INVALID. The first call on a
 * device looks up the array's device address, so make it before any stream capture. All calls
 * share the array: calls that overlap on the GPU (other streams or threads) race on it. The call
 * waits for its work to finish before it returns.
 * (No counterpart in the reference: merian's node always renders into graph-allocated images.) */
GBPT_API int gbpt_render_device_noalloc(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                        const gbpt_render_params* params, float* out_rgba_device);

/* ---- traversal queries (the GBuffer node's primary hit, and raw ray queries) ---------------
 * gbpt_trace_primary: the hit merian's GBuffer (Raytraced) node stores for each pixel
 * (gbuffer_rt.slang:18-58) with full-precision barycentrics and t, written to a host array of
 * width*height records. gbpt_trace: closest-hit (any_hit = 0) or occlusion (any_hit = 1, only
 * t is written: 0 = occluded, -1 = clear) for n device-resident rays. */
GBPT_API int gbpt_trace_primary(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                uint32_t width, uint32_t height, uint32_t instance_mask,
                                gbpt_hit* out_hits_host);
GBPT_API int gbpt_trace(gbpt_ctx* ctx, uint32_t scene, const gbpt_ray* rays_device, uint32_t n,
                        uint32_t instance_mask, int any_hit, gbpt_hit* hits_device);
/* Average CWBVH nodes visited and triangles tested per ray of the last gbpt_trace call made with
 * count_work = 1 (an instrumented traversal, used for the bytes-per-ray roofline). */
GBPT_API int gbpt_trace_counted(gbpt_ctx* ctx, uint32_t scene, const gbpt_ray* rays_device,
                                uint32_t n, uint32_t instance_mask, int any_hit,
                                gbpt_hit* hits_device, double* nodes_per_ray,
                                double* tris_per_ray);

/* ---- test hooks (device BSDF code run in isolation) ------------------------------------------
 * gbpt_debug_material_samples: n samples of a material at one shading point (incident direction
 * wi in the local shading frame, RNG PCG(pcg4d16(i, seed, 0, 0)) for sample i); 12 floats per
 * sample: wo.xyz, pdf, weight.rgb, valid, eval(wi, wo).rgb, pdf(wi, wo).
 * gbpt_debug_bsdf_check: merian's BSDF property checks (tests/bsdf/bsdf-checks.slang:30-135) on
 * the device BSDFs, one thread: kind 0 Lambert(albedo), 1 GGX(alpha, alpha_y), 2 conductor(alpha,
 * f0), 3 rough dielectric(alpha, eta, tint = albedo), 4 Fresnel mix GGX/Lambert(alpha, albedo,
 * ior_f0); 16 floats in the reference's slot layout. */
GBPT_API int gbpt_debug_material_samples(const gbpt_material* material, int front_facing,
                                         float ior, const float wi[3], uint32_t seed, uint32_t n,
                                         float* out_host);
GBPT_API int gbpt_debug_bsdf_check(int kind, const float wi[3], const float albedo[3],
                                   float alpha, float alpha_y, const float f0[3], float ior_f0,
                                   float eta, uint32_t n_samples, uint32_t seed, float* out16);
/* The primary shading point of each pixel as the render path caches it: 24 floats per pixel
 * (position, encoded face normal bits; shading normal, material id bits; tangent, flags bits
 * (1 = has material, 2 = front facing); bitangent, 0; emission, 0; ray direction, 0). */
GBPT_API int gbpt_debug_primary_points(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                       const gbpt_render_params* params, float* out_host);

/* ---- host helpers (no device work) ----------------------------------------------------------
 * Camera basis from look-at parameters (camera.cpp:263-266,349-367); vfov in radians. */
GBPT_API int gbpt_camera_look_at(const float position[3], const float target[3],
                                 const float up[3], float vfov, float aspect, float near_plane,
                                 float far_plane, gbpt_camera* out_camera);
GBPT_API uint32_t gbpt_encode_normal(const float n[3]);
GBPT_API uint32_t gbpt_pack_half2(float x, float y);

/* Seeded synthetic scenes (deterministic on any host; integer PCG32 and +-*÷√ only).
 * Cornell: unit box open at z=0, 5 walls of 8x8 cells, two rotated boxes of 4x4 cells per face,
 * 1,024 triangles, emissive 0.25x0.25 ceiling patch of radiance 15. Sizes are fixed: 1,024
 * triangles, 3,072 vertices, 8 geometries, 8 materials.
 * Soup: n triangles, centroids uniform in the unit cube, vertices at lognormal(ln 0.01, 0.5)
 * distances; n_geometries material groups split 60% Lambert / 30% GGX conductor / 10% GGX
 * dielectric. Vertices: 3n; geometries and materials: n_geometries.
 * Env: width x height RGBA32F sum of 8 Gaussian lobes. */
GBPT_API int gbpt_gen_cornell(uint64_t seed, gbpt_packed_vertex* vertices, uint32_t* indices,
                              gbpt_geometry* geometries, gbpt_material* materials);
GBPT_API int gbpt_gen_soup(uint64_t seed, uint32_t n_triangles, uint32_t n_geometries,
                           gbpt_packed_vertex* vertices, uint32_t* indices,
                           gbpt_geometry* geometries, gbpt_material* materials);
GBPT_API int gbpt_gen_env(uint64_t seed, uint32_t width, uint32_t height, float* texels);

#ifdef __cplusplus
}
#endif

#endif /* GBPT_H */

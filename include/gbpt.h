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

#define GBPT_ABI_VERSION 2u

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
/* Non-opaque geometry (merian: IsOpaque = 0x4 cleared, scene.hpp:46): every candidate hit runs the
 * material's alpha test (material-system.slang:28-38, scene.slang:500-519) and is skipped when the
 * alpha texture's alpha at the hit's uv is below 0.5. Off by default: geometry is opaque, as in
 * merian's ForceOpaque instances (scene.cpp:1849-1850). */
#define GBPT_MESH_ALPHA_TEST 0x100u

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
    int32_t alpha_texture;      /* -1 = none; its alpha channel is the alpha test's mask */
    uint32_t reserved[2];
} gbpt_material;

/* RGBA8 texture (a material's base_color_texture), sampled bilinearly with repeat addressing at
 * level 0 (merian's DefaultLODSampler); srgb = 1 decodes the colour channels from sRGB per texel
 * before filtering (an R8G8B8A8_SRGB image), 0 reads them as UNORM. */
typedef struct gbpt_texture {
    const uint8_t* texels; /* width*height*4 bytes, row-major, row 0 = v in [0, 1/height) */
    uint32_t width;
    uint32_t height;
    uint32_t srgb;
    uint32_t reserved;
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
    /* level 2, SIMT activity of those launches: warp-wide node steps and triangle-test steps,
     * and the lanes active in them (lanes / steps = active lanes of 32 per step) */
    uint64_t node_steps, node_lanes;
    uint64_t tri_steps, tri_lanes;
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

/* One texel of the GBuffer (Raytraced) node's outputs (gbuffer.slang:71-85 textures tex0..tex3,
 * plus gbuffer_rt.slang's emission output), 64 bytes. */
typedef struct gbpt_gbuffer_texel {
    uint32_t encoded_normal; /* tex0.x: shading normal, oct-encoded (encoding.slang:6-30) */
    uint32_t grad_z;         /* tex0.y: half2 depth change per pixel step in x and y */
    uint32_t instance_id;    /* tex1: PackedHitInfo (misses: all ids 0xFFFF...) */
    uint32_t primitive_id;
    uint16_t geometry_index;
    uint16_t instance_index;
    uint32_t barycentrics;   /* half2 */
    float motion[2];         /* tex2.xy: pixel-space motion vector */
    float linear_z;          /* tex2.z: |position - camera|, at most 65504 */
    float delta_z;           /* tex2.w */
    float albedo[3];         /* tex3.rgb: the BSDF's albedo toward the camera; on a miss the
                                environment radiance */
    float emission[3];       /* emitted radiance toward the camera */
} gbpt_gbuffer_texel;

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
 * Limits: spp at most the paths one pass over the array holds (228,908), a pixel
 * subset of at most 65,536 entries; larger requests return GBPT_ERR_INVALID. Every call looks up
 * the array's device address (no allocation; nothing cached, so a device reset between calls is
 * harmless); the first lookup on a device may load the library's module, so make the first call
 * on each device before any stream capture. All calls
 * share the array: calls that overlap on the GPU (other streams or threads) race on it. The call
 * waits for its work to finish before it returns.
 * (No counterpart in the reference: merian's node always renders into graph-allocated images.) */
GBPT_API int gbpt_render_device_noalloc(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                        const gbpt_render_params* params, float* out_rgba_device);

/* ---- batches and the request server ------------------------------------------------------
 * merian renders one request per graph iteration (Graph::run_node -> RenderPT::process,
 * graph.cpp:323-360); these calls have no counterpart there. They render many requests whose
 * paths share the wavefront's ticks (up to 8 Mi paths of whole pixels from up to 256 requests
 * per tick), so small requests fill the GPU together. Every result equals, bit for bit, what
 * gbpt_render / gbpt_render_device return for the request alone. */

/* One request: a scene, a camera, the node parameters (params.pixels is a host list, copied
 * during the call) and exactly one output, host or device (RGBA32F, one texel per pixel or per
 * listed pixel). */
typedef struct gbpt_request {
    uint32_t scene;
    uint32_t reserved;
    gbpt_camera camera;
    gbpt_render_params params;
    float* out_host;
    float* out_device;
} gbpt_request;

/* Renders n requests together and returns when every output is written. stats, when non-NULL,
 * sums over the batch. */
GBPT_API int gbpt_render_batch(gbpt_ctx* ctx, const gbpt_request* requests, uint32_t n,
                               gbpt_render_stats* stats);
/* gbpt_render_batch replays each tick from a captured CUDA graph (one per path length and
 * estimator) when enabled (1), or launches the kernels one by one (0, the default). */
GBPT_API int gbpt_set_graphs(gbpt_ctx* ctx, int enable);

/* The schedule of gbpt_render, gbpt_render_device and gbpt_render_batch. Outputs are the same
 * under every tuning, bit for bit: only the time changes. */
typedef struct gbpt_tuning {
    uint64_t wave_paths;    /* paths per tick: 0 = default (2^23), else in [1024, 2^24] */
    int32_t sort_materials; /* -1: as each request's params ask; 0 / 1: force off / on */
    int32_t use_graphs;     /* gbpt_render_batch replays ticks from CUDA graphs */
    int32_t bvh_build;      /* scenes created after it: GBPT_BVH_* */
    int32_t streams;        /* gbpt_render / gbpt_render_device: 2 (and 0, the default) = ticks
                               alternate between the context stream and a second stream with its
                               own work buffers, so one tick's last launches overlap the next
                               tick's first (not while profiling); 1 = ticks in order on the
                               context stream */
    /* warp scheduling of the persistent traversal launches, 0 = default each */
    int32_t trace_refill_lanes;   /* a warp refills its idle lanes with new rays once fewer than
                                     this many lanes are busy: [1, 32], default 20 */
    int32_t trace_postpone_lanes; /* a lane pushes its triangle group for later when fewer than
                                     this many lanes have triangles to test: [1, 32], default 6;
                                     closest-hit traversal only (a first-hit query tests its
                                     triangles at once) */
    int32_t trace_blocks_per_sm;  /* 128-thread blocks per SM of the traversal launches: [1, 64],
                                     capped at what is resident; default all resident */
} gbpt_tuning;

/* BVH build of gbpt_scene_create (the traversal finds the same hits in every case). */
#define GBPT_BVH_SPLIT 0  /* default: loose triangles split into up to 16 clipped references
                           * (single-level scenes), up to 4 for very loose ones (BLASes) */
#define GBPT_BVH_FAST 1   /* one reference per triangle: fastest build, smallest tree */
#define GBPT_BVH_MEDIUM 2 /* up to 4 references for very loose triangles only */

/* The traversal data gbpt_scene_create builds for a scene (replacing the driver's BLAS / TLAS
 * build, scene.cpp:1117-1120,1836-1882), built on the host alone, without a context or a device:
 * for inspection and host-side traversal (CPU walks of the same tree). nodes: 80-byte CWBVH
 * nodes (origin, exponents and inner-child mask; child and triangle bases; 8 meta bytes; 6 x 8
 * quantised child planes); tris: 48-byte triangle records (v0 + primitive id, v1 + geometry id,
 * v2 + flags: instance mask bits 0-7, two-sided bit 8, flip bit 9, alpha test bit 10), in leaf
 * order. For two-level scenes the top level comes first and a top-level record holds an
 * instance index. bvh_build is a GBPT_BVH_* value. The tree is the same on every host. */
typedef struct gbpt_bvh gbpt_bvh;
GBPT_API int gbpt_bvh_build(const gbpt_scene_desc* desc, int32_t bvh_build, gbpt_bvh** out);
GBPT_API int gbpt_bvh_info(const gbpt_bvh* bvh, const void** nodes, uint64_t* node_count,
                           const void** tris, uint64_t* tri_count, uint32_t* depth);
GBPT_API void gbpt_bvh_free(gbpt_bvh* bvh);

GBPT_API int gbpt_set_tuning(gbpt_ctx* ctx, const gbpt_tuning* tuning);
GBPT_API int gbpt_get_tuning(gbpt_ctx* ctx, gbpt_tuning* tuning);
/* Autotuner: renders the frame (camera, params: a whole frame, no pixel list) under candidate
 * schedules and keeps the fastest as the context's tuning, returning it. Stage 1: each tick size
 * (2^24 .. 2^21 paths, largest first; a smaller tick must be at least 2 % faster to be kept, since
 * larger ticks let more requests share one) with material sorting off and on (8 candidates,
 * ms_out in ascending tick size); then, from the best so far,
 * one parameter at a time: trace_refill_lanes in {12, 16, 20, 24, 28} (5), trace_postpone_lanes in
 * {2, 4, 6, 8, 12} (5), trace_blocks_per_sm in {6, 7, all resident} (3). ms_out, when non-NULL,
 * receives GBPT_AUTOTUNE_CANDIDATES times in that order (NaN for candidates not run). Results are
 * cached per (scene size, frame size, path length, estimator) bucket: a repeated call for the same
 * bucket applies the cached tuning without rendering. Outputs are discarded. */
#define GBPT_AUTOTUNE_CANDIDATES 32
GBPT_API int gbpt_autotune(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                           const gbpt_render_params* params, gbpt_tuning* out, double* ms_out);

/* The request server: one host thread per context admits submitted requests in arrival order
 * while their outputs fit a device arena reserved from free HBM at start, and renders the
 * admitted ones together, one tick after another (continuous batching: a request submitted while
 * others run joins the next tick). Scenes stay resident; a scene used by a queued or running
 * request cannot be destroyed (GBPT_ERR_BUSY). */
typedef struct gbpt_server_config {
    uint64_t wave_paths;  /* paths per tick (at most 2^24); 0 = the context's tuning, else 8 Mi.
                             The tuning's material-sort override, as at start, also applies */
    uint64_t arena_bytes; /* device arena for host-output staging and pixel lists;
                             0 = a quarter of the free HBM, at most 16 GiB */
    int32_t use_graphs;   /* replay ticks from captured CUDA graphs */
    uint32_t max_active;  /* requests admitted at once; 0 = 1024 */
} gbpt_server_config;

#define GBPT_REQ_QUEUED 0
#define GBPT_REQ_RUNNING 1
#define GBPT_REQ_DONE 2
#define GBPT_REQ_CANCELLED 3
#define GBPT_REQ_FAILED 4

typedef struct gbpt_request_status {
    int32_t state;   /* GBPT_REQ_* */
    int32_t error;   /* status code of a failed request */
    double submit_s; /* gbpt_clock() at submission, admission and completion */
    double admit_s;
    double done_s;
    uint64_t samples; /* pixels x spp */
} gbpt_request_status;

typedef struct gbpt_server_stats {
    uint64_t queued, active, completed;
    uint64_t ticks, kernel_launches, paths;
    uint64_t arena_bytes, wave_paths;
} gbpt_server_stats;

/* Seconds on the host's steady clock, the clock of gbpt_request_status. */
GBPT_API double gbpt_clock(void);
GBPT_API int gbpt_server_start(gbpt_ctx* ctx, const gbpt_server_config* config);
/* Cancels queued requests, finishes admitted ones and joins the server thread. */
GBPT_API int gbpt_server_stop(gbpt_ctx* ctx);
/* Queues a request; the caller keeps out_host / out_device valid until it has finished. */
GBPT_API int gbpt_server_submit(gbpt_ctx* ctx, const gbpt_request* request, uint64_t* ticket);
/* GBPT_OK when done, GBPT_ERR_BUSY while queued or running, GBPT_ERR_CANCELLED, or the error of a
 * failed request; status (optional) receives its state and timestamps. */
GBPT_API int gbpt_server_poll(gbpt_ctx* ctx, uint64_t ticket, gbpt_request_status* status);
/* As poll, after waiting up to timeout_s seconds (negative: without limit) for the request. */
GBPT_API int gbpt_server_wait(gbpt_ctx* ctx, uint64_t ticket, double timeout_s,
                              gbpt_request_status* status);
/* A queued request is dropped at once; a running one stops at the next tick boundary. */
GBPT_API int gbpt_server_cancel(gbpt_ctx* ctx, uint64_t ticket);
/* Forgets a finished request's record. */
GBPT_API int gbpt_server_release(gbpt_ctx* ctx, uint64_t ticket);
GBPT_API int gbpt_server_info(gbpt_ctx* ctx, gbpt_server_stats* stats);

/* ---- the nodes either side of the renderer ------------------------------------------------
 * Accumulate (accumulate.slang:233-257, static camera): per texel, when history > 0 and the
 * previous output is finite, n = min(history + 1, max_history), a = max(1 - alpha, 1/n),
 * out = out + a * (src - out), history = n; otherwise out = src, history = 1. With alpha = 1
 * and max_history = INFINITY (merian's gltf.json settings) out is the running mean of the
 * frames. RGBA32F device buffers of `texels` texels; history is one float per texel (zero, or
 * clear = 1, restarts). Enqueued on the context stream. */
GBPT_API int gbpt_accumulate(gbpt_ctx* ctx, const float* src_device, float* out_device,
                             float* history_device, uint64_t texels, float alpha,
                             float max_history, int clear);
/* Error Plot (error_to_buffer.slang): out8[0..3] = mean over texels of (reference - input)^2
 * per RGBA channel (MSE), out8[4..7] = mean |reference - input| (MAE), summed in double in a
 * fixed order. Synchronous. */
GBPT_API int gbpt_error_metrics(gbpt_ctx* ctx, const float* reference_device,
                                const float* input_device, uint64_t texels, double* out8);
/* Image Write / Image Read of PFM files (image_io.cpp:53-176): channels 1, 3 or 4 (RGBA is
 * written as RGB), top row first in memory, bottom row first in the file. gbpt_image_read_pfm
 * with texels = NULL returns the size only. Host only. */
GBPT_API int gbpt_image_write_pfm(const char* path, const float* texels, uint32_t width,
                                  uint32_t height, uint32_t channels);
GBPT_API int gbpt_image_read_pfm(const char* path, float* texels, uint32_t channels,
                                 uint32_t* width, uint32_t* height);
/* PNG to RGBA8 (the loaders' image textures): grey, RGB, palette, grey+alpha and RGBA, 8 and 16
 * bits (16-bit samples keep their high byte), not interlaced; top row first. rgba = NULL returns
 * the size only. Host only. */
GBPT_API int gbpt_image_read_png(const char* path, uint8_t* rgba, uint32_t* width,
                                 uint32_t* height);

/* ---- the node graph: merian graph JSONs of this path's nodes (graph.cpp) --------------------
 * merian's nodes are C++ classes behind a registry (node_registry.cpp:60-110) that Graph::run
 * calls once per iteration (graph.cpp:323-360). These calls host the same node types in C++:
 * "Render (Path-traced)", "GBuffer (Raytraced)", "Accumulate", "Image Write" (PFM), "Error
 * Plot", "GLTF Scene" and "PBRT Scene" (the loaders below; the scene is made resident when the
 * graph first runs), with merian's connector names, property keys and defaults, from a graph JSON in
 * merian's layout (examples/renderers/pt.json). A graph created with ctx = NULL is checked
 * (types, properties, edges) but cannot run. Not thread-safe: one caller per graph. Destroy a
 * graph before its context (its buffers and scene nodes' scenes live on that context).
 * Properties: gbpt_graph_set_property takes one JSON value ("group/key" for a property in a
 * group such as Image Write's "advanced") and returns merian's NodeStatusFlags (1 =
 * NEEDS_RECONNECT); unknown keys are errors there and warnings in the graph JSON. Outputs are
 * named "node.output" and read to the host (synchronising the context stream). */
typedef struct gbpt_graph gbpt_graph;
GBPT_API int gbpt_graph_create(gbpt_ctx* ctx, const char* graph_json, gbpt_graph** out_graph);
GBPT_API int gbpt_graph_destroy(gbpt_graph* graph);
/* nodes in run order (dependencies first, ties by name) */
GBPT_API int gbpt_graph_node_count(const gbpt_graph* graph, uint32_t* count);
GBPT_API int gbpt_graph_node(const gbpt_graph* graph, uint32_t index, const char** name,
                             const char** type);
GBPT_API uint32_t gbpt_graph_warning_count(const gbpt_graph* graph);
GBPT_API const char* gbpt_graph_warning(const gbpt_graph* graph, uint32_t index);
GBPT_API int gbpt_graph_set_property(gbpt_graph* graph, const char* node, const char* key,
                                     const char* json_value, uint32_t* out_flags);
/* The graph JSON's "cli" options (merian-graph-run, main.cpp:31-51): each names a JSON pointer
 * "/nodes/<node>/properties/<key>"; setting an option sets that property. Options whose pointer
 * names no property of an enabled node are dropped with a warning. */
GBPT_API int gbpt_graph_option(const gbpt_graph* graph, uint32_t index, const char** name,
                               const char** pointer);
GBPT_API int gbpt_graph_set_option(gbpt_graph* graph, const char* option, const char* json_value,
                                   uint32_t* out_flags);
/* key = NULL: every property of the node as one JSON object. length = the text's size. */
GBPT_API int gbpt_graph_get_property(const gbpt_graph* graph, const char* node, const char* key,
                                     char* json_out, uint64_t capacity, uint64_t* length);
/* Runs `iterations` graph iterations on the context stream. A node with a connected "scene"
 * input renders that scene with its file's camera; the others render `scene` with `camera`
 * (NULL when every renderer has a scene input). width x height is the extent of a renderer
 * without a GBuffer input. */
GBPT_API int gbpt_graph_run(gbpt_graph* graph, uint32_t scene, const gbpt_camera* camera,
                            uint32_t width, uint32_t height, uint32_t iterations);
/* The graph as a graph JSON in merian's layout (graph_load_store.cpp): "cli", then every node
 * with "enabled", "outputs", all "properties" and "type"; it loads back into the same graph. */
GBPT_API int gbpt_graph_to_json(const gbpt_graph* graph, char* json_out, uint64_t capacity,
                                uint64_t* length);
/* Checkpoint / resume of a progressive render: gbpt_graph_save writes directory/
 * graph_state.json (the iteration count, every node's properties and counters) and each
 * Accumulate node's image as PFM files (node.rgb.pfm = rgb, node.aux.pfm = (alpha, history, 0),
 * exact float32); gbpt_graph_load restores them into a graph made from the same JSON, and its
 * next run continues as if it had not stopped. JSON has no infinity: null stands for it. */
GBPT_API int gbpt_graph_save(gbpt_graph* graph, const char* directory);
GBPT_API int gbpt_graph_load(gbpt_graph* graph, const char* directory);
/* out_host = NULL returns the size only (floats_per_texel: 4 RGBA32F, 1 history, 16 GBuffer). */
GBPT_API int gbpt_graph_output(gbpt_graph* graph, const char* connector, float* out_host,
                               uint64_t capacity_floats, uint32_t* width, uint32_t* height,
                               uint32_t* floats_per_texel);

/* ---- traversal queries (the GBuffer node's primary hit, and raw ray queries) ---------------
 * gbpt_trace_primary: the hit merian's GBuffer (Raytraced) node stores for each pixel
 * (gbuffer_rt.slang:18-58) with full-precision barycentrics and t, written to a host array of
 * width*height records. gbpt_trace: closest-hit (any_hit = 0) or occlusion (any_hit = 1, only
 * t is written: 0 = occluded, -1 = clear) for n device-resident rays, on the context tuning's
 * traversal schedule (trace_* fields; with trace_postpone_lanes = 1 no triangle group is
 * postponed, so nodes and triangles are visited in the order of a one-ray-at-a-time walk). */
GBPT_API int gbpt_trace_primary(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                uint32_t width, uint32_t height, uint32_t instance_mask,
                                gbpt_hit* out_hits_host);
/* The GBuffer (Raytraced) node (gbuffer_rt.slang:18-94) on the same traversal: width*height
 * gbpt_gbuffer_texel in DEVICE memory, row-major, enqueued on the context stream. The camera is
 * static: motion vectors are 0. The albedo is what "demodulate albedo" divides out. */
GBPT_API int gbpt_gbuffer(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                          uint32_t width, uint32_t height, uint32_t instance_mask,
                          gbpt_gbuffer_texel* out_device);
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
/* Host-side fault injection for failure tests: the next `after` device allocations of the
 * library succeed, the `count` after them fail as if HBM were full (the call that needed them
 * returns GBPT_ERR_NO_MEMORY and leaves the context usable), then allocation is normal again;
 * count = 0 disarms. The allocation is refused before cudaMalloc is called: no GPU is involved. */
GBPT_API int gbpt_debug_fail_allocations(int64_t after, int64_t count);
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
/* The same box with every grid refined tess times per side: 1024 tess^2 triangles, 3 vertices per
 * triangle, 8 geometries and materials (tess in [1, 64]; tess = 1 is gbpt_gen_cornell). */
GBPT_API int gbpt_gen_cornell_tess(uint64_t seed, uint32_t tess, gbpt_packed_vertex* vertices,
                                   uint32_t* indices, gbpt_geometry* geometries,
                                   gbpt_material* materials);
GBPT_API int gbpt_gen_soup(uint64_t seed, uint32_t n_triangles, uint32_t n_geometries,
                           gbpt_packed_vertex* vertices, uint32_t* indices,
                           gbpt_geometry* geometries, gbpt_material* materials);
GBPT_API int gbpt_gen_env(uint64_t seed, uint32_t width, uint32_t height, float* texels);
/* A closed bumpy sphere for the instanced configuration: (n_u + 1) * n_v vertices (uv from the
 * latitude-longitude grid, smooth normals) and 2 * n_u * (n_v - 1) triangles. */
GBPT_API int gbpt_gen_blob(uint64_t seed, uint32_t n_u, uint32_t n_v, gbpt_packed_vertex* vertices,
                           uint32_t* indices);
/* A tileable sRGB value-noise RGBA8 texture, width * height * 4 bytes. */
GBPT_API int gbpt_gen_noise_texture(uint64_t seed, uint32_t width, uint32_t height, uint8_t* rgba);

/* ---- scene loader (merian PBRTScene, src/merian-shaders/scene/pbrt_scene.cpp) ----------------
 * gbpt_load_pbrt parses a pbrt-v4 scene file (Include/Import followed) into host arrays that
 * gbpt_loaded_scene_info exposes as a gbpt_scene_desc for gbpt_scene_create, with the file's
 * camera and film size. Shapes: trianglemesh, loopsubdiv (unsubdivided), plymesh (ASCII and
 * binary PLY), sphere, disk; materials: diffuse, coateddiffuse, conductor, coatedconductor,
 * dielectric, thindielectric, mix (the more probable side), others approximated as diffuse, as
 * merian converts them; diffuse area lights as emission; ObjectBegin/ObjectInstance as TLAS
 * instances; a constant infinite light as a uniform environment. Features it skips (image
 * textures and environments, other lights, media) are listed by gbpt_loaded_scene_warning. */
typedef struct gbpt_loaded_scene gbpt_loaded_scene;
typedef struct gbpt_loaded_info {
    gbpt_scene_desc desc; /* arrays owned by the loaded scene, valid until it is freed */
    gbpt_camera camera;   /* pbrt's perspective camera (fov on the shorter image axis) */
    uint32_t width;       /* Film xresolution (default 1280) */
    uint32_t height;      /* Film yresolution (default 720) */
    uint32_t warning_count;
    uint32_t reserved;
} gbpt_loaded_info;

GBPT_API int gbpt_load_pbrt(const char* path, gbpt_loaded_scene** out);
/* glTF 2.0 (.gltf with external or data-URI buffers, .glb) the way merian's GLTFScene reads it:
 * each mesh a BLAS, each node holding one a TLAS instance; triangle primitives with POSITION,
 * NORMAL, TEXCOORD_0, TANGENT; metallic-roughness materials mapped onto the OpenPBR record (base
 * colour factor x sRGB PNG texture, metallic, alpha = roughness^2, emissive x strength, ior,
 * transmission); non-OPAQUE alphaMode alpha-tested against the base colour texture; doubleSided
 * or transmissive -> two-sided; the first perspective camera. */
GBPT_API int gbpt_load_gltf(const char* path, gbpt_loaded_scene** out);
GBPT_API int gbpt_loaded_scene_info(const gbpt_loaded_scene* scene, gbpt_loaded_info* info);
/* Warning i (0 <= i < warning_count) of the load, or NULL. */
GBPT_API const char* gbpt_loaded_scene_warning(const gbpt_loaded_scene* scene, uint32_t i);
GBPT_API void gbpt_loaded_scene_free(gbpt_loaded_scene* scene);

#ifdef __cplusplus
}
#endif

#endif /* GBPT_H */

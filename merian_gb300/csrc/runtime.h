// Internal interface between the C ABI (api.cpp, host only) and the kernels (kernels.cu).
#pragma once

#include "gbpt.h"

#include <cstdint>
#include <cuda_runtime.h>
#include <string>
#include <vector>

namespace gbpt {

struct DevScene; // device_scene.cuh

// GBPT_TRI_AXIS_COPIES: each traversal triangle record is stored three times, its vertices'
// coordinates permuted for each dominant ray axis kz to (kz + 1, kz + 2, kz) mod 3, so the
// watertight test reads the ray's frame from memory instead of selecting 9 coordinates at run
// time. Copy c of record i is record c n + i of the uploaded array (n records), so a ray reads
// one contiguous copy. 0: one copy, coordinates selected at run time.
#ifndef GBPT_TRI_AXIS_COPIES
#define GBPT_TRI_AXIS_COPIES 1
#endif
constexpr int kTriCopies = GBPT_TRI_AXIS_COPIES ? 3 : 1;

// GBPT_ENV_ALIAS: next-event estimation picks the environment texel by alias tables (a row, then
// a column: two dependent loads) instead of inverting the marginal and conditional CDFs (a
// guide-table lookup and a short search each)
#ifndef GBPT_ENV_ALIAS
#define GBPT_ENV_ALIAS 1
#endif

// A scene resident in HBM. All pointers are device pointers owned by the context.
struct SceneGPU {
    void* nodes = nullptr;      // CWBVH, 80 B per node
    void* tris = nullptr;       // 48 B per triangle record and copy (kTriCopies)
    void* verts = nullptr;      // gbpt_packed_vertex
    void* idx = nullptr;        // uint32 x 3 per triangle
    // the three vertices of each triangle in one 80-byte record (20 words: vertex k at word 6k,
    // 8 bytes of padding), by triangle index; null when geometries that share a triangle range
    // disagree on its first vertex
    void* tri_verts = nullptr;
    void* geoms = nullptr;      // GeomGPU
    void* geom_key = nullptr;   // uint8 material-sort key per geometry
    void* mats = nullptr;       // gbpt_material
    void* env = nullptr;        // float4 texels
    void* env_marg = nullptr;
    void* env_cond = nullptr;
    void* env_func = nullptr;
    void* light_tris = nullptr; // 3 float4 per emissive triangle
    void* light_cdf = nullptr;
    // guide tables of the CDFs (upper bound of k / G for k = 0..G, G a power of two)
    void* light_guide = nullptr;
    void* env_marg_guide = nullptr;
    void* env_cond_guide = nullptr; // G + 1 entries per row
    // GBPT_ENV_ALIAS: alias tables of the same density, uint2 (keep probability bits, alias) per
    // row and per texel
    void* env_rows = nullptr;
    void* env_cols = nullptr;
    uint32_t light_g = 0, env_marg_g = 0, env_cond_g = 0;
    uint64_t n_nodes = 0, n_tris = 0, n_verts = 0;
    uint32_t geom_count = 0, mat_count = 0;
    uint32_t ew = 0, eh = 0;
    float env_m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    float env_intensity = 1.0f;
    float env_func_int = 0.0f;
    uint32_t n_lights = 0;
    float light_total = 0.0f;
    // two-level scenes: 7 float4 per instance (object-to-world and world-to-object rows, BLAS
    // root / mask / first geometry); the TLAS is the first tree of `nodes`, its leaves the first
    // records of `tris`
    void* inst = nullptr;
    uint32_t n_inst = 0;
    // RGBA8 textures
    void* tex = nullptr;
    void* tex_info = nullptr; // uint4 per texture: first texel, width, height, sRGB
    void* srgb_lut = nullptr; // 256 floats
    uint32_t n_tex = 0;
    bool alpha = false; // some geometry is alpha-tested (GBPT_MESH_ALPHA_TEST)
    uint32_t depth = 0;
    uint64_t bytes = 0;
};

// Work buffers of the wavefront, grown on demand and kept for the context's lifetime.
// cudaMalloc behind the host-side fault injection of gbpt_debug_fail_allocations (api.cpp). On
// failure *p is null.
cudaError_t device_malloc(void** p, size_t bytes);

struct Work {
    uint64_t path_cap = 0;  // paths per wave
    uint64_t pixel_cap = 0; // pixels per wave
    // true when the buffers are carved from memory the Work does not own: they are never grown
    // or freed, and a wave never exceeds path_cap
    bool fixed = false;
    // path state (SoA, indexed by wave-local path id)
    // 2 float4 per path, one 32-byte sector: (throughput rgb, current IOR), (radiance rgb, pdf
    // of the last BSDF sample)
    float4* path = nullptr;
    // ray queues (two, ping-pong): 2 float4 per entry, one 32-byte sector: (origin, the path's
    // RNG state bits), (direction, entry tag bits: chunk << 24 | path); every bounce ray spans
    // [0, kRayTmax], and the path's RNG state travels with its ray
    float4* q_od[2] = {nullptr, nullptr};
    // closest hit per queue entry, 2 uint4 (one sector): (t, u, v, primitive), (geometry,
    // instance of two-level hits or 0xFFFFFFFF, 0, 0)
    uint4* hit = nullptr;
    // shadow queue
    float4* s_od = nullptr;     // 2 float4 per entry: (o, tmax), (d, 0)
    float4* s_contrib = nullptr;
    uint32_t* s_path = nullptr;
    // material-sorted shading: key per queue entry and the sorted order (absent in fixed Work)
    uint8_t* keys = nullptr;
    uint32_t* perm = nullptr;
    // per-pixel primary shading point cache (kPixFloat4 float4 per pixel)
    float4* pix = nullptr;
    uint32_t* pix_id = nullptr; // pixel ids of the current request (device)
    uint64_t pix_id_cap = 0;
    float4* out = nullptr;      // device output staging for host-output renders
    uint64_t out_cap = 0;
    // counters: [0],[1] queue counts, [2] shadow count, [3] error flags, [4],[5] fetch cursors,
    // [8..11] material-key counts, [12..15] their scatter cursors
    uint32_t* counters = nullptr;
    unsigned long long* stats = nullptr; // [0] rays, [1] shadow rays, [2] closest-hit rays
    // request, scene and tick tables of the batch being rendered
    void* tables = nullptr;
    uint64_t tables_bytes = 0;
    uint64_t bytes = 0;
    // changes (to a value never used before, process-wide) whenever a buffer is (re)allocated:
    // CUDA graphs captured over older buffers are then recaptured
    uint64_t generation = 0;
};

// One request of a batch: a scene, a camera, the render parameters and a device output of
// pixel_count float4 (mean rgb, mean squared luminance), indexed like the pixel list.
struct BatchItem {
    const SceneGPU* scene = nullptr;
    gbpt_camera camera{};
    gbpt_render_params params{};
    const uint32_t* pixels_device = nullptr; // nullptr: all pixels, row-major
    uint32_t pixel_count = 0;
    float4* out_device = nullptr;
};

// Paths per wave: 8 Mi paths keep ~1.5 GB of path state and queues resident.
constexpr uint64_t kWavePaths = 1ull << 23;
// float4 per pixel of the primary shading point cache: position + encoded face normal, frame
// (n + material, t + flags, b + demodulation r), emission + demodulation g, ray direction +
// demodulation b, base colour texture
constexpr uint64_t kPixFloat4 = 7;

// Optional per-kernel timing (CUDA events around each launch) and traversal work counters.
struct Profile {
    int level = 0; // 0 off, 1 kernel timing, 2 timing + CWBVH nodes / triangles per ray
    std::vector<cudaEvent_t> ev; // start/end pairs
    std::vector<int> cls;        // launch class of each pair: 0 trace, 1 shade, 2 shadow, 3 other
    size_t used = 0;
    int begin(cudaStream_t st, int c);
    void end(cudaStream_t st, int pair);
    void reset() { used = 0; cls.clear(); }
    void destroy();
};

struct RenderArgs {
    gbpt_camera camera;
    gbpt_render_params params;
    const uint32_t* pixels_device; // nullptr: all pixels
    uint32_t pixel_count;
    float4* out_device;
};

// A request as the tick engine sees it: its pixels are scheduled in list order, whole pixels
// per tick; cursor counts the pixels already scheduled.
struct TickItem : BatchItem {
    uint32_t cursor = 0;
};

// Warp scheduling of the persistent traversal kernels, chosen at launch (gbpt_tuning, searched
// by the autotuner; results never depend on it): a warp leaves its traversal loop to refill its
// idle lanes with new rays once fewer than refill_lanes lanes are busy; a lane pushes its
// triangle group for later when fewer than postpone_lanes lanes of the warp have triangles to
// test; the closest-hit and any-hit launches run blocks_per_sm blocks of 128 threads per SM
// (0: every block that is resident at once).
struct TraceSched {
    uint32_t refill_lanes = 20;
    uint32_t postpone_lanes = 6;
    uint32_t blocks_per_sm = 0;
};

// Plans ticks over requests, uploads each tick's tables and enqueues its kernels on one stream
// (wavefront.cu). A tick is at most `wave` paths of whole pixels from up to 256 requests.
struct TickEngine {
    Work* work = nullptr;
    cudaStream_t stream = nullptr;
    uint64_t wave = kWavePaths;
    TraceSched sched;
    // replay each tick shape (path length, NEE) from a captured CUDA graph; needs a stream that
    // can be captured, and keeps a whole wave of work buffers
    bool use_graphs = false;
    // internal
    struct Graph {
        uint32_t shape;
        cudaGraphExec_t exec;
        uint64_t launches;
    };
    std::vector<Graph> graphs;
    uint64_t graph_generation = 0; // Work::generation the graphs were captured with
    std::vector<unsigned char> stage;
    std::vector<const SceneGPU*> scene_ptrs;
    int grids[7] = {0, 0, 0, 0, 0, 0, 0}; // launch grids, computed at the first tick
    void release(); // destroys the graphs
};

// Enqueues the next tick over items (earlier items first; a request is never overtaken by a later
// one). *n_paths = 0 when no item has pixels left. `done` receives the indices of the items whose
// last pixels are in this tick: their outputs are final once the tick has run. work_ctr (device,
// >= 2 counters) receives traversal work when prof->level >= 2.
int tick_enqueue(TickEngine& e, TickItem* const* items, uint32_t n_items, uint64_t* n_paths,
                 std::vector<uint32_t>* done, uint64_t* launches, Profile* prof,
                 unsigned long long* work_ctr);
// Renders every item (ticks until all pixels are scheduled); results are independent of the
// other items in the batch, bit for bit.
// With e2, ticks alternate between e (even) and e2 (odd; its own stream and work buffers):
// e2's stream starts after `fork` is recorded on e's, and e's waits for `join` recorded on e2's.
int render_batch(TickEngine& e, const BatchItem* items, uint32_t n_items, uint64_t* launches,
                 Profile* prof, unsigned long long* work_ctr, TickEngine* e2 = nullptr,
                 cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);
// wave: paths per tick, 0 = kWavePaths. With work2, ticks alternate between stream (even) and
// stream2 (odd, over work2): stream2 starts after `fork` is recorded on stream, and stream waits
// for `join` recorded on stream2 at the end.
int render_frame(const SceneGPU& scene, Work& work, const RenderArgs& args, cudaStream_t stream,
                 uint64_t* launches, Profile* prof, unsigned long long* work_ctr,
                 uint64_t wave = 0, Work* work2 = nullptr, cudaStream_t stream2 = nullptr,
                 cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr,
                 const TraceSched& sched = TraceSched{});
int primary_points(const SceneGPU& scene, Work& work, const RenderArgs& args, cudaStream_t stream,
                   float* out_device);
// Bytes of tick tables for ticks of at most max_chunks requests.
uint64_t tick_table_bytes(uint32_t max_chunks);
int num_sms();

// Rendering from the library's fixed scratch array (kernels.cu): no allocation, synchronous.
constexpr uint64_t kStaticScratchBytes = 64ull << 20;
constexpr uint32_t kStaticMaxPixelList = 1u << 16;
uint64_t static_scratch_paths();
int render_frame_static(const SceneGPU& scene, const RenderArgs& args, const uint32_t* pixels_host,
                        cudaStream_t stream, std::string& err);
int trace_rays(const SceneGPU& scene, const gbpt_ray* rays, uint32_t n, uint32_t mask, int any_hit,
               gbpt_hit* hits, unsigned long long* counters_device, cudaStream_t stream,
               const TraceSched& sched = TraceSched{});
int trace_primary(const SceneGPU& scene, const gbpt_camera& cam, uint32_t w, uint32_t h,
                  uint32_t mask, gbpt_hit* hits_device, uint32_t* err_device, cudaStream_t stream);
int gbuffer(const SceneGPU& scene, const gbpt_camera& cam, uint32_t w, uint32_t h, uint32_t mask,
            gbpt_gbuffer_texel* out_device, uint32_t* err_device, cudaStream_t stream);
int work_reserve(Work& work, uint64_t paths, uint64_t pixels);
void work_free(Work& work);

std::string cuda_error_string(cudaError_t e);

} // namespace gbpt

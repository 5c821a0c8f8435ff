// C ABI of the GB300 path tracer (declared in include/gbpt.h): context, scene upload, render,
// batches and traversal queries. Host-only C++ on the CUDA runtime; the kernels live in
// wavefront.cu and kernels.cu, the request server in server.cpp.
#include "context.h"
#include "gbpt.h"
#include "host_common.h"
#include "runtime.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace gbpt {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

struct GeomHost {
    uint32_t first_vertex, first_triangle, material, flags;
};
static_assert(sizeof(GeomHost) == 16, "GeomGPU layout");

int check_ctx(gbpt_ctx* ctx) {
    if (!ctx) {
        set_error("null context");
        return GBPT_ERR_INVALID;
    }
    const cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
        set_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        return GBPT_ERR_CUDA;
    }
    return GBPT_OK;
}

double host_clock() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

} // namespace gbpt

namespace gbpt {
std::mutex g_inject_mu;
int64_t g_inject_after = 0, g_inject_count = 0; // see gbpt_debug_fail_allocations

cudaError_t device_malloc(void** p, size_t bytes) {
    {
        std::lock_guard<std::mutex> lk(g_inject_mu);
        if (g_inject_count > 0) {
            if (g_inject_after > 0) {
                --g_inject_after;
            } else {
                --g_inject_count;
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
        }
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) *p = nullptr;
    return e;
}
TraceSched sched_of(const gbpt_tuning& t) {
    TraceSched s;
    if (t.trace_refill_lanes > 0) s.refill_lanes = (uint32_t)t.trace_refill_lanes;
    if (t.trace_postpone_lanes > 0) s.postpone_lanes = (uint32_t)t.trace_postpone_lanes;
    if (t.trace_blocks_per_sm > 0) s.blocks_per_sm = (uint32_t)t.trace_blocks_per_sm;
    return s;
}
} // namespace gbpt

using namespace gbpt;

namespace {

int upload(void** dst, const void* src, size_t bytes, uint64_t& total) {
    if (bytes == 0) {
        *dst = nullptr;
        return GBPT_OK;
    }
    GBPT_CUDA_CHECK(device_malloc(dst, bytes));
    total += bytes;
    const cudaError_t e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(*dst);
        *dst = nullptr;
        set_error(std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        return GBPT_ERR_CUDA;
    }
    return GBPT_OK;
}

// Inverse of a row-major 3x4 affine transform (double); false when singular.
bool invert_affine(const float* m, double* inv) {
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9],
                 i = m[10];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double det = a * A + b * B + c * C;
    if (!(std::fabs(det) > 1e-30) || !std::isfinite(det)) return false;
    const double r[9] = {A / det, -(b * i - c * h) / det, (b * f - c * e) / det,
                         B / det, (a * i - c * g) / det,  -(a * f - c * d) / det,
                         C / det, -(a * h - b * g) / det, (a * e - b * d) / det};
    const double t[3] = {m[3], m[7], m[11]};
    for (int row = 0; row < 3; ++row) {
        inv[4 * row + 0] = r[3 * row + 0];
        inv[4 * row + 1] = r[3 * row + 1];
        inv[4 * row + 2] = r[3 * row + 2];
        inv[4 * row + 3] = -(r[3 * row + 0] * t[0] + r[3 * row + 1] * t[1] + r[3 * row + 2] * t[2]);
    }
    return true;
}

void free_scene(SceneGPU& s) {
    void* ptrs[] = {s.nodes,    s.tris,     s.verts,      s.idx,       s.tri_verts, s.geoms,    s.mats,
                    s.env,      s.env_marg, s.env_cond,   s.env_func,  s.light_tris, s.light_cdf,
                    s.light_guide, s.env_marg_guide, s.env_cond_guide, s.env_rows, s.env_cols,
                    s.geom_key,
                    s.inst,     s.tex,      s.tex_info,   s.srgb_lut};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    s = SceneGPU{};
}

// Guide table of an increasing float CDF a[0..n) ending at 1: entry k (k = 0..G) is
// upper_bound(a, a + n, k / G) with the device's float comparison; G is the power of two at or
// above n, at most 4096 (k / G and u * G are exact in float).
std::vector<uint32_t> cdf_guide(const float* a, uint32_t n, uint32_t& G) {
    G = 1;
    while (G < n && G < 4096u) G <<= 1;
    std::vector<uint32_t> g(G + 1);
    for (uint32_t k = 0; k <= G; ++k)
        g[k] = (uint32_t)(std::upper_bound(a, a + n, (float)k / (float)G) - a);
    return g;
}

// GBPT_SHADE_TRI_RECORDS: upload the de-indexed per-triangle vertex records read by shading
#ifndef GBPT_SHADE_TRI_RECORDS
#define GBPT_SHADE_TRI_RECORDS 1
#endif

// The build input's reference splitting for a GBPT_BVH_* setting. GBPT_BVH_SPLIT splits hard in
// single-level scenes (measured on the 1M-triangle soup: ratio 2 / depth 4 renders 25 % faster
// than no splitting) and lightly in the BLASes of two-level scenes (instanced meshes: ratio 8 /
// depth 2 is 5 % faster than none, ratio 2 / depth 4 5 % slower).
#ifndef GBPT_BVH_SPLIT_RATIO
#define GBPT_BVH_SPLIT_RATIO 2.0
#endif
#ifndef GBPT_BVH_SPLIT_DEPTH
#define GBPT_BVH_SPLIT_DEPTH 4
#endif
#ifndef GBPT_BVH_BLAS_SPLIT_RATIO
#define GBPT_BVH_BLAS_SPLIT_RATIO 8.0
#endif
#ifndef GBPT_BVH_BLAS_SPLIT_DEPTH
#define GBPT_BVH_BLAS_SPLIT_DEPTH 2
#endif
void set_split(BuildInput& in, int32_t bvh_build, bool blas) {
    in.split = bvh_build != GBPT_BVH_FAST;
    if (bvh_build == GBPT_BVH_MEDIUM || blas) {
        in.split_ratio = GBPT_BVH_BLAS_SPLIT_RATIO;
        in.split_depth = GBPT_BVH_BLAS_SPLIT_DEPTH;
    } else {
        in.split_ratio = GBPT_BVH_SPLIT_RATIO;
        in.split_depth = GBPT_BVH_SPLIT_DEPTH;
    }
}

// Reads and clears the kernels' error words (the context's work buffers, the second tick
// stream's, and the per-ray entry points'); returns GBPT_ERR_DEVICE when one was set. The
// second stream's ticks have joined the context stream before any caller gets here.
int check_device_error(gbpt_ctx* ctx) {
    uint32_t flags[3] = {0, 0, 0};
    if (ctx->work.counters) {
        GBPT_CUDA_CHECK(cudaMemcpyAsync(&flags[0], ctx->work.counters + 3, 4,
                                        cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (ctx->work2.counters) {
        GBPT_CUDA_CHECK(cudaMemcpyAsync(&flags[2], ctx->work2.counters + 3, 4,
                                        cudaMemcpyDeviceToHost, ctx->stream));
    }
    unsigned long long misc = 0;
    GBPT_CUDA_CHECK(cudaMemcpyAsync(&misc, ctx->d_misc + 2, 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBPT_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    flags[1] = (uint32_t)misc;
    if (flags[0] | flags[1] | flags[2]) {
        if (ctx->work.counters) cudaMemsetAsync(ctx->work.counters + 3, 0, 4, ctx->stream);
        if (ctx->work2.counters) cudaMemsetAsync(ctx->work2.counters + 3, 0, 4, ctx->stream);
        cudaMemsetAsync(ctx->d_misc + 2, 0, 8, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        set_error("kernel error flag raised (traversal stack overflow)");
        return GBPT_ERR_DEVICE;
    }
    return GBPT_OK;
}

} // namespace

extern "C" {

GBPT_API uint32_t gbpt_abi_version(void) { return GBPT_ABI_VERSION; }

GBPT_API const char* gbpt_last_error(void) { return g_last_error.c_str(); }

GBPT_API int gbpt_create(int device, uint64_t stream, gbpt_ctx** out_ctx) {
    if (!out_ctx) {
        set_error("gbpt_create: null out_ctx");
        return GBPT_ERR_INVALID;
    }
    *out_ctx = nullptr;
    int n = 0;
    GBPT_CUDA_CHECK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) {
        set_error("gbpt_create: no such CUDA device");
        return GBPT_ERR_INVALID;
    }
    GBPT_CUDA_CHECK(cudaSetDevice(device));
    auto ctx = std::make_unique<gbpt_ctx>();
    ctx->device = device;
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        GBPT_CUDA_CHECK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    GBPT_CUDA_CHECK(device_malloc((void**)&ctx->d_misc, 8 * sizeof(unsigned long long)));
    GBPT_CUDA_CHECK(cudaMemset(ctx->d_misc, 0, 8 * sizeof(unsigned long long)));
    GBPT_CUDA_CHECK(cudaEventCreate(&ctx->ev0));
    GBPT_CUDA_CHECK(cudaEventCreate(&ctx->ev1));
    const int rc = work_reserve(ctx->work, 0, 0);
    if (rc != GBPT_OK) {
        set_error("gbpt_create: work buffer allocation failed");
        return rc;
    }
    *out_ctx = ctx.release();
    return GBPT_OK;
}

GBPT_API int gbpt_destroy(gbpt_ctx* ctx) {
    if (!ctx) return GBPT_OK;
    cudaSetDevice(ctx->device);
    server_shutdown(ctx->server);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->scenes) free_scene(kv.second);
    ctx->batch.release();
    ctx->batch2.release();
    work_free(ctx->work);
    if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
    work_free(ctx->work2);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    ctx->prof.destroy();
    if (ctx->d_misc) cudaFree(ctx->d_misc);
    if (ctx->d_hits) cudaFree(ctx->d_hits);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GBPT_OK;
}

GBPT_API int gbpt_synchronize(gbpt_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    GBPT_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

GBPT_API int gbpt_memory_info(gbpt_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes,
                              uint64_t* ctx_bytes) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    size_t f = 0, t = 0;
    GBPT_CUDA_CHECK(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    if (ctx_bytes) {
        std::lock_guard<std::mutex> lk(ctx->mu);
        uint64_t b = ctx->work.bytes;
        for (auto& kv : ctx->scenes) b += kv.second.bytes;
        *ctx_bytes = b;
    }
    return GBPT_OK;
}

GBPT_API int gbpt_debug_fail_allocations(int64_t after, int64_t count) {
    if (after < 0 || count < 0) {
        set_error("gbpt_debug_fail_allocations: negative argument");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(gbpt::g_inject_mu);
    gbpt::g_inject_after = after;
    gbpt::g_inject_count = count;
    return GBPT_OK;
}

GBPT_API int gbpt_set_profiling(gbpt_ctx* ctx, int level) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (level < 0 || level > 2) {
        set_error("gbpt_set_profiling: level must be 0, 1 or 2");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->prof.level = level;
    return GBPT_OK;
}

// Validates a scene description and builds its traversal data on the host: the CWBVH (the top
// level over the instances first, then every BLAS, for two-level scenes) and the instance records
// (28 floats each). Shared by gbpt_scene_create and gbpt_bvh_build.
static int build_scene_bvh(const gbpt_scene_desc* d, int32_t bvh_build, CwBvh& bvh,
                           std::vector<float>& inst_rec) {
    int rc = GBPT_OK;
    if (!d || (d->triangle_count && (!d->vertices || !d->indices)) ||
        (d->geometry_count && !d->geometries) || (d->material_count && !d->materials)) {
        set_error("gbpt_scene_create: null pointer in scene description");
        return GBPT_ERR_INVALID;
    }
    const bool two_level = d->instance_count != 0;
    if (two_level) {
        if (!d->instances || !d->blas_ranges || d->blas_count == 0) {
            set_error("gbpt_scene_create: instances need BLAS ranges");
            return GBPT_ERR_INVALID;
        }
        for (uint32_t b = 0; b < d->blas_count; ++b) {
            const gbpt_blas_range& r = d->blas_ranges[b];
            if (r.geometry_count == 0 ||
                (uint64_t)r.first_geometry + r.geometry_count > d->geometry_count) {
                set_error("gbpt_scene_create: BLAS " + std::to_string(b) + " geometry range out of bounds");
                return GBPT_ERR_INVALID;
            }
        }
        for (uint32_t i = 0; i < d->instance_count; ++i) {
            const gbpt_instance& in = d->instances[i];
            bool finite = in.blas < d->blas_count;
            for (float x : in.object_to_world) finite = finite && std::isfinite(x);
            double inv[12];
            if (!finite || !invert_affine(in.object_to_world, inv)) {
                set_error("gbpt_scene_create: instance " + std::to_string(i) +
                          " has a bad BLAS index or a singular / non-finite transform");
                return GBPT_ERR_INVALID;
            }
        }
    }
    for (uint32_t t = 0; t < d->texture_count; ++t) {
        const gbpt_texture& tx = d->textures[t];
        if (!tx.texels || tx.width == 0 || tx.height == 0 ||
            (uint64_t)tx.width * tx.height > (1ull << 28)) {
            set_error("gbpt_scene_create: texture " + std::to_string(t) + " is empty or too large");
            return GBPT_ERR_INVALID;
        }
    }
    // validate geometry ranges and gather world-space triangles
    BuildInput bi;
    set_split(bi, bvh_build, false);
    uint64_t total_tris = 0;
    for (uint32_t g = 0; g < d->geometry_count; ++g) {
        const gbpt_geometry& geo = d->geometries[g];
        if ((uint64_t)geo.first_triangle + geo.triangle_count > d->triangle_count) {
            set_error("gbpt_scene_create: geometry " + std::to_string(g) + " triangle range out of bounds");
            return GBPT_ERR_INVALID;
        }
        if (geo.material_id >= d->material_count) {
            set_error("gbpt_scene_create: geometry " + std::to_string(g) + " material out of range");
            return GBPT_ERR_INVALID;
        }
        total_tris += geo.triangle_count;
    }
    if (total_tris >= (1ull << 31)) {
        set_error("gbpt_scene_create: too many triangles");
        return GBPT_ERR_INVALID;
    }
    for (uint32_t m = 0; m < d->material_count; ++m) {
        if (d->materials[m].model > GBPT_MATERIAL_OPENPBR_TRANSMISSION) {
            set_error("gbpt_scene_create: material " + std::to_string(m) + " has an unknown model");
            return GBPT_ERR_INVALID;
        }
    }
    // triangles of the given geometries (object space for a BLAS), vertex indices checked
    auto gather = [&](uint32_t g_first, uint32_t g_count, BuildInput& in) -> int {
        for (uint32_t g = g_first; g < g_first + g_count; ++g) {
            const gbpt_geometry& geo = d->geometries[g];
            const uint32_t tf = (geo.instance_mask & 0xFFu) |
                                ((geo.flags & GBPT_MESH_TWO_SIDED) ? (1u << 8) : 0u) |
                                ((geo.flags & GBPT_MESH_FLIP_FACING) ? (1u << 9) : 0u) |
                                ((geo.flags & GBPT_MESH_ALPHA_TEST) ? (1u << 10) : 0u);
            for (uint32_t k = 0; k < geo.triangle_count; ++k) {
                const uint64_t tri = (uint64_t)geo.first_triangle + k;
                for (int c = 0; c < 3; ++c) {
                    const uint64_t vi = (uint64_t)geo.first_vertex + d->indices[3 * tri + c];
                    if (vi >= d->vertex_count) {
                        set_error("gbpt_scene_create: vertex index out of bounds in geometry " +
                                  std::to_string(g));
                        return GBPT_ERR_INVALID;
                    }
                    const float* p = d->vertices[vi].position;
                    if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2])) {
                        set_error("gbpt_scene_create: non-finite vertex position");
                        return GBPT_ERR_INVALID;
                    }
                    in.v.insert(in.v.end(), p, p + 3);
                }
                in.prim.push_back(k);
                in.geom.push_back(g);
                in.flags.push_back(tf);
            }
        }
        return GBPT_OK;
    };
    if (!two_level) {
        bi.v.reserve(9 * total_tris);
        bi.prim.reserve(total_tris);
        bi.geom.reserve(total_tris);
        bi.flags.reserve(total_tris);
        if ((rc = gather(0, d->geometry_count, bi))) return rc;
        // each tree level puts at most one node group and one postponed triangle group on the
        // 48-entry traversal stack
        if (!build_cwbvh(bi, bvh, 24)) return GBPT_ERR_INVALID;
    } else {
        // one CWBVH per BLAS in object space, a top-level CWBVH over the instances' world boxes
        // (a leaf record per instance: its index and mask), concatenated top level first; the
        // stack holds both levels, so their depths share the 24 levels
        std::vector<CwBvh> blas(d->blas_count);
        for (uint32_t b = 0; b < d->blas_count; ++b) {
            BuildInput in;
            set_split(in, bvh_build, true);
            if ((rc = gather(d->blas_ranges[b].first_geometry, d->blas_ranges[b].geometry_count, in)))
                return rc;
            if (in.prim.empty()) {
                set_error("gbpt_scene_create: BLAS " + std::to_string(b) + " has no triangles");
                return GBPT_ERR_INVALID;
            }
            if (!build_cwbvh(in, blas[b], 16)) return GBPT_ERR_INVALID;
        }
        BuildInput top;
        for (uint32_t i = 0; i < d->instance_count; ++i) {
            const gbpt_instance& in = d->instances[i];
            const CwBvh& b = blas[in.blas];
            double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int c = 0; c < 8; ++c) {
                const double p[3] = {(c & 1) ? b.hi[0] : b.lo[0], (c & 2) ? b.hi[1] : b.lo[1],
                                     (c & 4) ? b.hi[2] : b.lo[2]};
                for (int a = 0; a < 3; ++a) {
                    const float* r = in.object_to_world + 4 * a;
                    const double w = (double)r[0] * p[0] + (double)r[1] * p[1] +
                                     (double)r[2] * p[2] + (double)r[3];
                    lo[a] = std::min(lo[a], w);
                    hi[a] = std::max(hi[a], w);
                }
            }
            // a degenerate triangle spanning the box (its bounds are the box, its centroid the
            // box centre); rounded outward to float
            float flo[3], fhi[3], fc[3];
            for (int a = 0; a < 3; ++a) {
                flo[a] = std::nextafter((float)lo[a], -INFINITY);
                fhi[a] = std::nextafter((float)hi[a], INFINITY);
                fc[a] = 0.5f * (flo[a] + fhi[a]);
            }
            top.v.insert(top.v.end(), flo, flo + 3);
            top.v.insert(top.v.end(), fhi, fhi + 3);
            top.v.insert(top.v.end(), fc, fc + 3);
            top.prim.push_back(i);
            top.geom.push_back(0);
            top.flags.push_back(in.mask & 0xFFu);
        }
        if (!build_cwbvh(top, bvh, 8)) return GBPT_ERR_INVALID;
        uint32_t max_blas_depth = 0;
        std::vector<uint32_t> root(d->blas_count);
        for (uint32_t b = 0; b < d->blas_count; ++b) {
            const uint32_t node_off = (uint32_t)bvh.nodes.size(), tri_off = (uint32_t)bvh.tris.size();
            root[b] = node_off;
            for (CwNode nd : blas[b].nodes) {
                nd.w[4] += node_off; // child base
                nd.w[5] += tri_off;  // triangle base
                bvh.nodes.push_back(nd);
            }
            bvh.tris.insert(bvh.tris.end(), blas[b].tris.begin(), blas[b].tris.end());
            max_blas_depth = std::max(max_blas_depth, blas[b].depth);
        }
        bvh.depth += max_blas_depth;
        for (uint32_t i = 0; i < d->instance_count; ++i) {
            const gbpt_instance& in = d->instances[i];
            double inv[12];
            invert_affine(in.object_to_world, inv);
            float rec[28];
            for (int k = 0; k < 12; ++k) rec[k] = in.object_to_world[k];
            for (int k = 0; k < 12; ++k) rec[12 + k] = (float)inv[k];
            const uint32_t bits[4] = {root[in.blas], in.mask & 0xFFu,
                                      d->blas_ranges[in.blas].first_geometry, 0u};
            std::memcpy(&rec[24], bits, 16);
            inst_rec.insert(inst_rec.end(), rec, rec + 28);
        }
    }
    return GBPT_OK;
}

} // extern "C"

struct gbpt_bvh {
    gbpt::CwBvh bvh;
    std::vector<float> inst_rec;
};

extern "C" {

GBPT_API int gbpt_bvh_build(const gbpt_scene_desc* d, int32_t bvh_build, gbpt_bvh** out) {
    if (!out) {
        set_error("gbpt_bvh_build: null output");
        return GBPT_ERR_INVALID;
    }
    *out = nullptr;
    if (bvh_build < GBPT_BVH_SPLIT || bvh_build > GBPT_BVH_MEDIUM) {
        set_error("gbpt_bvh_build: bvh_build must be a GBPT_BVH_* value");
        return GBPT_ERR_INVALID;
    }
    auto b = std::make_unique<gbpt_bvh>();
    const int rc = build_scene_bvh(d, bvh_build, b->bvh, b->inst_rec);
    if (rc) return rc;
    *out = b.release();
    return GBPT_OK;
}

GBPT_API int gbpt_bvh_info(const gbpt_bvh* b, const void** nodes, uint64_t* node_count,
                           const void** tris, uint64_t* tri_count, uint32_t* depth) {
    if (!b) {
        set_error("gbpt_bvh_info: null bvh");
        return GBPT_ERR_INVALID;
    }
    if (nodes) *nodes = b->bvh.nodes.data();
    if (node_count) *node_count = b->bvh.nodes.size();
    if (tris) *tris = b->bvh.tris.data();
    if (tri_count) *tri_count = b->bvh.tris.size();
    if (depth) *depth = b->bvh.depth;
    return GBPT_OK;
}

GBPT_API void gbpt_bvh_free(gbpt_bvh* b) { delete b; }

GBPT_API int gbpt_scene_create(gbpt_ctx* ctx, const gbpt_scene_desc* d, uint32_t* out_scene) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out_scene) {
        set_error("gbpt_scene_create: null out_scene");
        return GBPT_ERR_INVALID;
    }
    const bool two_level = d && d->instance_count != 0;
    CwBvh bvh;
    std::vector<float> inst_rec; // 28 floats per instance
    if ((rc = build_scene_bvh(d, ctx->tuning.bvh_build, bvh, inst_rec))) return rc;

    SceneGPU s;
    std::lock_guard<std::mutex> lk(ctx->mu);
    uint64_t bytes = 0;
    auto fail = [&](int code) {
        free_scene(s);
        return code;
    };
    if ((rc = upload(&s.nodes, bvh.nodes.data(), bvh.nodes.size() * sizeof(CwNode), bytes))) return fail(rc);
#if GBPT_TRI_AXIS_COPIES
    {
        // three copies of the records, one after the other, coordinates in the order
        // (c + 1, c + 2, c) mod 3 in copy c (the traversal's watertight test reads copy kz)
        std::vector<TriRecord> rec(3 * bvh.tris.size());
        for (size_t i = 0; i < bvh.tris.size(); ++i) {
            const TriRecord& r = bvh.tris[i];
            for (int c = 0; c < 3; ++c) {
                TriRecord& o = rec[c * bvh.tris.size() + i];
                o = r;
                for (int a = 0; a < 3; ++a) {
                    const int src = (c + 1 + a) % 3;
                    o.v0[a] = r.v0[src];
                    o.v1[a] = r.v1[src];
                    o.v2[a] = r.v2[src];
                }
            }
        }
        if ((rc = upload(&s.tris, rec.data(), rec.size() * sizeof(TriRecord), bytes))) return fail(rc);
    }
#else
    if ((rc = upload(&s.tris, bvh.tris.data(), bvh.tris.size() * sizeof(TriRecord), bytes))) return fail(rc);
#endif
    if ((rc = upload(&s.verts, d->vertices, d->vertex_count * sizeof(gbpt_packed_vertex), bytes))) return fail(rc);
    if ((rc = upload(&s.idx, d->indices, d->triangle_count * 3 * sizeof(uint32_t), bytes))) return fail(rc);
#if GBPT_SHADE_TRI_RECORDS
    // the vertices of each triangle in one record, so shading reads one 80-byte run instead of an
    // index triple and then three vertices; kept only when every triangle has one first vertex
    if (d->triangle_count) {
        constexpr uint32_t kUnset = 0xFFFFFFFFu;
        std::vector<uint32_t> fv(d->triangle_count, kUnset);
        bool unique = true;
        for (uint32_t g = 0; g < d->geometry_count && unique; ++g) {
            const gbpt_geometry& geo = d->geometries[g];
            for (uint32_t k = 0; k < geo.triangle_count; ++k) {
                uint32_t& f = fv[(uint64_t)geo.first_triangle + k];
                if (f != kUnset && f != geo.first_vertex) {
                    unique = false;
                    break;
                }
                f = geo.first_vertex;
            }
        }
        if (unique) {
            std::vector<uint32_t> rec(20ull * d->triangle_count, 0u);
            for (uint64_t t = 0; t < d->triangle_count; ++t) {
                if (fv[t] == kUnset) continue;
                for (int c = 0; c < 3; ++c) {
                    // a geometry outside every BLAS of a two-level scene is never traversed and
                    // its indices were not checked: such a vertex stays zero
                    const uint64_t vi = (uint64_t)fv[t] + d->indices[3 * t + c];
                    if (vi < d->vertex_count)
                        std::memcpy(&rec[20 * t + 6 * c], &d->vertices[vi], sizeof(gbpt_packed_vertex));
                }
            }
            if ((rc = upload(&s.tri_verts, rec.data(), rec.size() * sizeof(uint32_t), bytes))) return fail(rc);
        }
    }
#endif
    std::vector<GeomHost> gh(d->geometry_count);
    for (uint32_t g = 0; g < d->geometry_count; ++g)
        gh[g] = {d->geometries[g].first_vertex, d->geometries[g].first_triangle,
                 d->geometries[g].material_id, d->geometries[g].flags};
    if ((rc = upload(&s.geoms, gh.data(), gh.size() * sizeof(GeomHost), bytes))) return fail(rc);
    if ((rc = upload(&s.mats, d->materials, d->material_count * sizeof(gbpt_material), bytes))) return fail(rc);
    // material-sort key per geometry: 0 environment (UseEnvMap), 1 + min(model, 2) otherwise
    {
        std::vector<uint8_t> keys(std::max<uint32_t>(d->geometry_count, 1u), 0u);
        for (uint32_t g = 0; g < d->geometry_count; ++g) {
            const gbpt_geometry& geo = d->geometries[g];
            if (!(geo.flags & GBPT_MESH_USE_ENV_MAP))
                keys[g] = (uint8_t)(1u + std::min(d->materials[geo.material_id].model, 2u));
        }
        if ((rc = upload(&s.geom_key, keys.data(), keys.size(), bytes))) return fail(rc);
    }
    if (two_level) {
        if ((rc = upload(&s.inst, inst_rec.data(), inst_rec.size() * sizeof(float), bytes))) return fail(rc);
        s.n_inst = d->instance_count;
    }
    s.n_nodes = bvh.nodes.size();
    s.n_tris = bvh.tris.size();
    s.n_verts = d->vertex_count;
    s.geom_count = d->geometry_count;
    s.mat_count = d->material_count;
    s.depth = bvh.depth;

    // emissive triangles, power = area x luminance (next-event estimation)
    {
        std::vector<float> lt;
        std::vector<double> pw;
        // every placement of a geometry: once in a single-level scene, once per instance of
        // its BLAS (world-space copies) in a two-level scene
        std::vector<std::pair<uint32_t, const float*>> placements;
        if (!two_level) {
            for (uint32_t g = 0; g < d->geometry_count; ++g) placements.push_back({g, nullptr});
        } else {
            for (uint32_t i = 0; i < d->instance_count; ++i) {
                const gbpt_blas_range& r = d->blas_ranges[d->instances[i].blas];
                for (uint32_t g = r.first_geometry; g < r.first_geometry + r.geometry_count; ++g)
                    placements.push_back({g, d->instances[i].object_to_world});
            }
        }
        for (const auto& pl : placements) {
            const uint32_t g = pl.first;
            const gbpt_geometry& geo = d->geometries[g];
            const gbpt_material& m = d->materials[geo.material_id];
            if (m.model == GBPT_MATERIAL_DIFFUSE) continue;
            const double lum = 0.299 * m.emission[0] + 0.587 * m.emission[1] + 0.114 * m.emission[2];
            if (!(lum > 0.0)) continue;
            for (uint32_t k = 0; k < geo.triangle_count; ++k) {
                const uint64_t tri = (uint64_t)geo.first_triangle + k;
                float pw_[3][3];
                const float* p[3];
                for (int c = 0; c < 3; ++c) {
                    const float* q = d->vertices[geo.first_vertex + d->indices[3 * tri + c]].position;
                    if (pl.second) { // to world space
                        for (int a = 0; a < 3; ++a) {
                            const float* r = pl.second + 4 * a;
                            pw_[c][a] = (float)((double)r[0] * q[0] + (double)r[1] * q[1] +
                                                (double)r[2] * q[2] + (double)r[3]);
                        }
                        p[c] = pw_[c];
                    } else {
                        p[c] = q;
                    }
                }
                const double e1[3] = {(double)p[1][0] - p[0][0], (double)p[1][1] - p[0][1], (double)p[1][2] - p[0][2]};
                const double e2[3] = {(double)p[2][0] - p[0][0], (double)p[2][1] - p[0][1], (double)p[2][2] - p[0][2]};
                const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                             cz = e1[0] * e2[1] - e1[1] * e2[0];
                const double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
                if (!(area > 0.0)) continue;
                pw.push_back(area * lum);
                uint32_t gw = g, fw = (geo.flags & GBPT_MESH_FLIP_FACING) ? 1u : 0u, zw = 0;
                float f[12];
                for (int c = 0; c < 3; ++c) {
                    f[4 * c + 0] = p[c][0];
                    f[4 * c + 1] = p[c][1];
                    f[4 * c + 2] = p[c][2];
                }
                std::memcpy(&f[3], &gw, 4);
                std::memcpy(&f[7], &fw, 4);
                std::memcpy(&f[11], &zw, 4);
                lt.insert(lt.end(), f, f + 12);
            }
        }
        if (!pw.empty()) {
            double acc = 0.0;
            for (double x : pw) acc += x;
            std::vector<float> cdf(pw.size());
            double run = 0.0;
            for (size_t i = 0; i < pw.size(); ++i) {
                run += pw[i];
                cdf[i] = (float)(run / acc);
            }
            cdf.back() = 1.0f;
            if ((rc = upload(&s.light_tris, lt.data(), lt.size() * sizeof(float), bytes))) return fail(rc);
            if ((rc = upload(&s.light_cdf, cdf.data(), cdf.size() * sizeof(float), bytes))) return fail(rc);
            const std::vector<uint32_t> lg = cdf_guide(cdf.data(), (uint32_t)cdf.size(), s.light_g);
            if ((rc = upload(&s.light_guide, lg.data(), lg.size() * 4, bytes))) return fail(rc);
            s.n_lights = (uint32_t)pw.size();
            s.light_total = (float)acc;
        }
    }
    // environment and its importance-sampling tables (luminance x sin(theta), floored)
    if (d->env && d->env->texels && d->env->width && d->env->height) {
        const gbpt_env_map& e = *d->env;
        const uint32_t w = e.width, h = e.height;
        if ((rc = upload(&s.env, e.texels, (size_t)w * h * 4 * sizeof(float), bytes))) return fail(rc);
        s.ew = w;
        s.eh = h;
        std::memcpy(s.env_m, e.to_local, sizeof(s.env_m));
        s.env_intensity = e.intensity;
        std::vector<double> func((size_t)w * h);
        double mean = 0.0;
        for (uint32_t y = 0; y < h; ++y) {
            const double st = std::sin(3.14159265358979323846 * (y + 0.5) / h);
            for (uint32_t x = 0; x < w; ++x) {
                const float* t = &e.texels[4 * ((size_t)y * w + x)];
                const double l = std::max(0.0, 0.299 * t[0] + 0.587 * t[1] + 0.114 * t[2]);
                func[(size_t)y * w + x] = l * st;
                mean += l * st;
            }
        }
        mean /= (double)w * h;
        for (double& f : func) f += 1e-3 * mean + 1e-30;
        std::vector<float> ffunc(func.size()), cond((size_t)h * (w + 1)), marg(h + 1);
        std::vector<double> rows(h);
        double tot = 0.0;
        for (uint32_t y = 0; y < h; ++y) {
            double r = 0.0;
            cond[(size_t)y * (w + 1)] = 0.0f;
            for (uint32_t x = 0; x < w; ++x) r += func[(size_t)y * w + x];
            double run = 0.0;
            for (uint32_t x = 0; x < w; ++x) {
                run += func[(size_t)y * w + x];
                cond[(size_t)y * (w + 1) + x + 1] = (float)(run / r);
            }
            cond[(size_t)y * (w + 1) + w] = 1.0f;
            rows[y] = r;
            tot += r;
        }
        double run = 0.0;
        marg[0] = 0.0f;
        for (uint32_t y = 0; y < h; ++y) {
            run += rows[y];
            marg[y + 1] = (float)(run / tot);
        }
        marg[h] = 1.0f;
        for (size_t i = 0; i < func.size(); ++i) ffunc[i] = (float)func[i];
        s.env_func_int = (float)(tot / ((double)w * h));
#if GBPT_ENV_ALIAS
        {
            // the same density by alias tables: the row by the row sums, then the column in it
            std::vector<uint32_t> at(2 * (size_t)h), ct(2 * (size_t)w * h);
            alias_table(rows.data(), h, at.data());
            for (uint32_t y = 0; y < h; ++y)
                alias_table(&func[(size_t)y * w], w, &ct[2 * (size_t)y * w]);
            if ((rc = upload(&s.env_rows, at.data(), at.size() * 4, bytes))) return fail(rc);
            if ((rc = upload(&s.env_cols, ct.data(), ct.size() * 4, bytes))) return fail(rc);
        }
#endif
        if ((rc = upload(&s.env_func, ffunc.data(), ffunc.size() * sizeof(float), bytes))) return fail(rc);
#if !GBPT_ENV_ALIAS
        if ((rc = upload(&s.env_cond, cond.data(), cond.size() * sizeof(float), bytes))) return fail(rc);
        if ((rc = upload(&s.env_marg, marg.data(), marg.size() * sizeof(float), bytes))) return fail(rc);
        const std::vector<uint32_t> mg = cdf_guide(marg.data() + 1, h, s.env_marg_g);
        std::vector<uint32_t> cg;
        for (uint32_t y = 0; y < h; ++y) {
            const std::vector<uint32_t> row =
                cdf_guide(cond.data() + (size_t)y * (w + 1) + 1, w, s.env_cond_g);
            cg.insert(cg.end(), row.begin(), row.end());
        }
        if ((rc = upload(&s.env_marg_guide, mg.data(), mg.size() * 4, bytes))) return fail(rc);
        if ((rc = upload(&s.env_cond_guide, cg.data(), cg.size() * 4, bytes))) return fail(rc);
#endif
    }
    // RGBA8 textures, concatenated, with (first texel, width, height, sRGB) per texture and the
    // sRGB decoding table (IEC 61966-2-1), evaluated in double and rounded once
    if (d->texture_count) {
        std::vector<uint32_t> info;
        uint64_t total = 0;
        for (uint32_t t = 0; t < d->texture_count; ++t) {
            const gbpt_texture& tx = d->textures[t];
            info.insert(info.end(), {(uint32_t)total, tx.width, tx.height, tx.srgb ? 1u : 0u});
            total += (uint64_t)tx.width * tx.height;
        }
        if (total >= (1ull << 32)) {
            set_error("gbpt_scene_create: textures too large");
            return fail(GBPT_ERR_INVALID);
        }
        std::vector<uint8_t> texels(total * 4);
        for (uint32_t t = 0; t < d->texture_count; ++t) {
            const gbpt_texture& tx = d->textures[t];
            std::memcpy(texels.data() + (size_t)info[4 * t] * 4, tx.texels,
                        (size_t)tx.width * tx.height * 4);
        }
        float lut[256];
        for (int i = 0; i < 256; ++i) {
            const double c = i / 255.0;
            lut[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        if ((rc = upload(&s.tex, texels.data(), texels.size(), bytes))) return fail(rc);
        if ((rc = upload(&s.tex_info, info.data(), info.size() * 4, bytes))) return fail(rc);
        if ((rc = upload(&s.srgb_lut, lut, sizeof(lut), bytes))) return fail(rc);
        s.n_tex = d->texture_count;
    }
    for (uint32_t g = 0; g < d->geometry_count; ++g)
        s.alpha |= (d->geometries[g].flags & GBPT_MESH_ALPHA_TEST) != 0u;
    s.bytes = bytes;
    const uint32_t id = ctx->next_scene++;
    ctx->scenes[id] = s;
    *out_scene = id;
    return GBPT_OK;
}

GBPT_API int gbpt_scene_destroy(gbpt_ctx* ctx, uint32_t scene) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_scene_destroy: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    auto users = ctx->scene_users.find(scene);
    if (users != ctx->scene_users.end() && users->second > 0) {
        set_error("gbpt_scene_destroy: the scene is used by queued or running server requests");
        return GBPT_ERR_BUSY;
    }
    GBPT_CUDA_CHECK(cudaStreamSynchronize(ctx->stream)); // work in flight may still read it
    free_scene(it->second);
    ctx->scenes.erase(it);
    return GBPT_OK;
}

GBPT_API int gbpt_scene_stats(gbpt_ctx* ctx, uint32_t scene, uint64_t* nodes, uint64_t* tris,
                              uint64_t* bytes, uint32_t* depth) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_scene_stats: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    if (nodes) *nodes = it->second.n_nodes;
    if (tris) *tris = it->second.n_tris;
    if (bytes) *bytes = it->second.bytes;
    if (depth) *depth = it->second.depth;
    return GBPT_OK;
}

} // extern "C"

int gbpt::validate_params(const gbpt_camera* cam, const gbpt_render_params* p) {
    if (!cam || !p) {
        set_error("null camera or params");
        return GBPT_ERR_INVALID;
    }
    if (p->width == 0 || p->height == 0 || (uint64_t)p->width * p->height > (1ull << 31)) {
        set_error("render: width/height out of range");
        return GBPT_ERR_INVALID;
    }
    if (p->spp < 0 || p->spp > (1 << 24) || p->max_path_length < 1 || p->max_path_length > 64) {
        set_error("render: spp must be in [0, 2^24] and max path length in [1, 64]");
        return GBPT_ERR_INVALID;
    }
    if (p->pixel_count && !p->pixels) {
        set_error("render: pixel_count without a pixel list");
        return GBPT_ERR_INVALID;
    }
    for (uint32_t i = 0; i < p->pixel_count; ++i) {
        if (p->pixels[i] >= p->width * p->height) {
            set_error("render: pixel id out of range");
            return GBPT_ERR_INVALID;
        }
    }
    return GBPT_OK;
}

extern "C" {

static int read_stats(gbpt_ctx* ctx, uint64_t samples, uint64_t launches, Profile* prof,
                      gbpt_render_stats* stats, bool two);
// Whether this render alternates its ticks over two streams (gbpt_tuning.streams 0 or 2, not
// while profiling): creates the second stream, its events and work counters at first use.
static int use_two_streams(gbpt_ctx* ctx, const Profile* prof, bool* two) {
    *two = false;
    if (ctx->tuning.streams == 1 || prof) return GBPT_OK;
    if (!ctx->stream2 &&
        cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking) != cudaSuccess) {
        ctx->stream2 = nullptr;
        set_error("render: cannot create the second tick stream");
        return GBPT_ERR_CUDA;
    }
    for (cudaEvent_t* e : {&ctx->ev_fork, &ctx->ev_join}) {
        if (!*e && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
            *e = nullptr;
            set_error("render: cannot create the tick stream events");
            return GBPT_ERR_CUDA;
        }
    }
    const int rc = work_reserve(ctx->work2, 0, 0);
    if (rc != GBPT_OK) {
        set_error("render: work buffer allocation failed");
        return rc;
    }
    *two = true;
    return GBPT_OK;
}

static int render_impl(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* cam,
                       const gbpt_render_params* p, float* out_dev, float* out_host,
                       gbpt_render_stats* stats) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = validate_params(cam, p))) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("render: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    Work& w = ctx->work;
    const uint32_t n_pix = p->pixel_count ? p->pixel_count : p->width * p->height;
    RenderArgs a;
    a.camera = *cam;
    a.params = *p;
    if (ctx->tuning.sort_materials >= 0) a.params.sort_materials = ctx->tuning.sort_materials;
    a.pixel_count = n_pix;
    a.pixels_device = nullptr;
    if (p->pixel_count) {
        if (p->pixel_count > w.pix_id_cap) {
            if (w.pix_id) cudaFree(w.pix_id);
            w.pix_id = nullptr;
            w.pix_id_cap = 0;
            GBPT_CUDA_CHECK(device_malloc((void**)&w.pix_id, (size_t)p->pixel_count * 4));
            w.pix_id_cap = p->pixel_count;
        }
        GBPT_CUDA_CHECK(cudaMemcpyAsync(w.pix_id, p->pixels, (size_t)p->pixel_count * 4,
                                        cudaMemcpyHostToDevice, ctx->stream));
        a.pixels_device = w.pix_id;
    }
    if (!out_dev) {
        if (n_pix > w.out_cap) {
            if (w.out) cudaFree(w.out);
            w.out = nullptr;
            w.out_cap = 0;
            GBPT_CUDA_CHECK(device_malloc((void**)&w.out, (size_t)n_pix * sizeof(float4)));
            w.out_cap = n_pix;
        }
        a.out_device = w.out;
    } else {
        a.out_device = (float4*)out_dev;
    }
    if (p->spp == 0) {
        GBPT_CUDA_CHECK(cudaMemsetAsync(a.out_device, 0, (size_t)n_pix * sizeof(float4), ctx->stream));
    }
    uint64_t launches = 0;
    Profile* prof = stats && ctx->prof.level > 0 ? &ctx->prof : nullptr;
    if (stats) {
        GBPT_CUDA_CHECK(cudaMemsetAsync(w.stats, 0, 4 * sizeof(unsigned long long), ctx->stream));
        GBPT_CUDA_CHECK(cudaMemsetAsync(ctx->d_misc, 0, 2 * sizeof(unsigned long long), ctx->stream));
        GBPT_CUDA_CHECK(cudaMemsetAsync(ctx->d_misc + 4, 0, 4 * sizeof(unsigned long long),
                                        ctx->stream));
        GBPT_CUDA_CHECK(cudaEventRecord(ctx->ev0, ctx->stream));
        if (prof) prof->reset();
    }
    // a tuned tick holds at least one whole pixel
    const uint64_t wave = ctx->tuning.wave_paths
                              ? std::max<uint64_t>(ctx->tuning.wave_paths, (uint64_t)p->spp)
                              : 0;
    bool two = false;
    if ((rc = use_two_streams(ctx, prof, &two)) != GBPT_OK) return rc;
    if (two && stats)
        GBPT_CUDA_CHECK(cudaMemsetAsync(ctx->work2.stats, 0, 4 * sizeof(unsigned long long),
                                        ctx->stream));
    const TraceSched sched = sched_of(ctx->tuning);
    rc = two ? render_frame(it->second, w, a, ctx->stream, &launches, prof, ctx->d_misc, wave,
                            &ctx->work2, ctx->stream2, ctx->ev_fork, ctx->ev_join, sched)
             : render_frame(it->second, w, a, ctx->stream, &launches, prof, ctx->d_misc, wave,
                            nullptr, nullptr, nullptr, nullptr, sched);
    if (rc != GBPT_OK) {
        set_error(rc == GBPT_ERR_NO_MEMORY ? "render: work buffer allocation failed"
                                           : "render: kernel launch failed: " +
                                                 cuda_error_string(cudaGetLastError()));
        return rc;
    }
    if (stats) GBPT_CUDA_CHECK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (out_host) {
        GBPT_CUDA_CHECK(cudaMemcpyAsync(out_host, a.out_device, (size_t)n_pix * sizeof(float4),
                                        cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (stats || out_host) {
        if ((rc = check_device_error(ctx))) return rc;
    }
    if (stats)
        return read_stats(ctx, (uint64_t)n_pix * (uint64_t)p->spp, launches, prof, stats, two);
    return GBPT_OK;
}

// Fills stats after a synchronised render: device counters, the event pair ev0/ev1 and, when
// profiling, the per-class kernel times.
static int read_stats(gbpt_ctx* ctx, uint64_t samples, uint64_t launches, Profile* prof,
                      gbpt_render_stats* stats, bool two) {
    Work& w = ctx->work;
    {
        unsigned long long st[3] = {0, 0, 0}, wk[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        GBPT_CUDA_CHECK(cudaMemcpy(st, w.stats, sizeof(st), cudaMemcpyDeviceToHost));
        if (two) {
            unsigned long long st2[3] = {0, 0, 0};
            GBPT_CUDA_CHECK(cudaMemcpy(st2, ctx->work2.stats, sizeof(st2), cudaMemcpyDeviceToHost));
            for (int k = 0; k < 3; ++k) st[k] += st2[k];
        }
        GBPT_CUDA_CHECK(cudaMemcpy(wk, ctx->d_misc, sizeof(wk), cudaMemcpyDeviceToHost));
        float ms = 0.f;
        GBPT_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        std::memset(stats, 0, sizeof(*stats));
        stats->samples = samples;
        stats->rays = st[0];
        stats->shadow_rays = st[1];
        stats->trace_rays = st[2];
        stats->kernel_launches = launches;
        stats->device_ms = ms;
        if (prof) {
            double cls_ms[4] = {0, 0, 0, 0};
            for (size_t i = 0; i < prof->used; ++i) {
                float t = 0.f;
                GBPT_CUDA_CHECK(cudaEventElapsedTime(&t, prof->ev[2 * i], prof->ev[2 * i + 1]));
                cls_ms[prof->cls[i]] += t;
                if (prof->cls[i] == 0) stats->trace_launches++;
            }
            stats->trace_ms = cls_ms[0];
            stats->shade_ms = cls_ms[1];
            stats->shadow_ms = cls_ms[2];
            stats->other_ms = cls_ms[3];
            if (prof->level >= 2) {
                stats->nodes_visited = wk[0];
                stats->tris_tested = wk[1];
                stats->node_steps = wk[4];
                stats->node_lanes = wk[5];
                stats->tri_steps = wk[6];
                stats->tri_lanes = wk[7];
            }
        }
    }
    return GBPT_OK;
}

GBPT_API int gbpt_render(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                         const gbpt_render_params* params, float* out_rgba_host,
                         gbpt_render_stats* stats) {
    if (!out_rgba_host) {
        set_error("gbpt_render: null output");
        return GBPT_ERR_INVALID;
    }
    return render_impl(ctx, scene, camera, params, nullptr, out_rgba_host, stats);
}

GBPT_API int gbpt_render_device(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                const gbpt_render_params* params, float* out_rgba_device,
                                gbpt_render_stats* stats) {
    if (!out_rgba_device) {
        set_error("gbpt_render_device: null output");
        return GBPT_ERR_INVALID;
    }
    return render_impl(ctx, scene, camera, params, out_rgba_device, nullptr, stats);
}

// Render through the library's fixed scratch array: no device allocation on this path.
GBPT_API int gbpt_render_device_noalloc(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                        const gbpt_render_params* p, float* out_rgba_device) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = validate_params(camera, p))) return rc;
    if (!out_rgba_device) {
        set_error("gbpt_render_device_noalloc: null output");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_render_device_noalloc: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    const uint32_t n_pix = p->pixel_count ? p->pixel_count : p->width * p->height;
    if (p->spp == 0) {
        GBPT_CUDA_CHECK(cudaMemsetAsync(out_rgba_device, 0, (size_t)n_pix * sizeof(float4),
                                        ctx->stream));
        GBPT_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        return GBPT_OK;
    }
    RenderArgs a;
    a.camera = *camera;
    a.params = *p;
    a.pixel_count = n_pix;
    a.pixels_device = nullptr;
    a.out_device = (float4*)out_rgba_device;
    std::string err;
    rc = render_frame_static(it->second, a, p->pixel_count ? p->pixels : nullptr, ctx->stream, err);
    if (rc != GBPT_OK) set_error("gbpt_render_device_noalloc: " + err);
    return rc;
}

// Many requests through the context's tick engine: their paths share ticks.
GBPT_API int gbpt_render_batch(gbpt_ctx* ctx, const gbpt_request* reqs, uint32_t n,
                               gbpt_render_stats* stats) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (n && !reqs) {
        set_error("gbpt_render_batch: null request array");
        return GBPT_ERR_INVALID;
    }
    uint64_t list_words = 0, host_texels = 0, samples = 0;
    for (uint32_t i = 0; i < n; ++i) {
        if ((rc = validate_params(&reqs[i].camera, &reqs[i].params))) return rc;
        if (!reqs[i].out_host == !reqs[i].out_device) {
            set_error("gbpt_render_batch: request " + std::to_string(i) +
                      " needs exactly one of out_host and out_device");
            return GBPT_ERR_INVALID;
        }
        const gbpt_render_params& p = reqs[i].params;
        const uint64_t np = p.pixel_count ? p.pixel_count : (uint64_t)p.width * p.height;
        list_words += p.pixel_count;
        if (reqs[i].out_host) host_texels += np;
        samples += np * (uint64_t)p.spp;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::vector<BatchItem> items(n);
    for (uint32_t i = 0; i < n; ++i) {
        auto it = ctx->scenes.find(reqs[i].scene);
        if (it == ctx->scenes.end()) {
            set_error("gbpt_render_batch: request " + std::to_string(i) + ": unknown scene id");
            return GBPT_ERR_NOT_FOUND;
        }
        items[i].scene = &it->second;
    }
    // pixel lists and host outputs go through the context's staging buffers
    Work& w = ctx->work;
    if (list_words > w.pix_id_cap) {
        if (w.pix_id) cudaFree(w.pix_id);
        w.pix_id = nullptr;
        w.pix_id_cap = 0;
        GBPT_CUDA_CHECK(device_malloc((void**)&w.pix_id, (size_t)list_words * 4));
        w.pix_id_cap = list_words;
    }
    if (host_texels > w.out_cap) {
        if (w.out) cudaFree(w.out);
        w.out = nullptr;
        w.out_cap = 0;
        GBPT_CUDA_CHECK(device_malloc((void**)&w.out, (size_t)host_texels * sizeof(float4)));
        w.out_cap = host_texels;
    }
    uint64_t list_at = 0, out_at = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const gbpt_render_params& p = reqs[i].params;
        const uint32_t np = p.pixel_count ? p.pixel_count : p.width * p.height;
        items[i].camera = reqs[i].camera;
        items[i].params = reqs[i].params;
        if (ctx->tuning.sort_materials >= 0)
            items[i].params.sort_materials = ctx->tuning.sort_materials;
        items[i].pixel_count = np;
        items[i].pixels_device = nullptr;
        if (p.pixel_count) {
            GBPT_CUDA_CHECK(cudaMemcpyAsync(w.pix_id + list_at, p.pixels, (size_t)p.pixel_count * 4,
                                            cudaMemcpyHostToDevice, ctx->stream));
            items[i].pixels_device = w.pix_id + list_at;
            list_at += p.pixel_count;
        }
        if (reqs[i].out_host) {
            items[i].out_device = w.out + out_at;
            out_at += np;
        } else {
            items[i].out_device = (float4*)reqs[i].out_device;
        }
        if (p.spp == 0)
            GBPT_CUDA_CHECK(cudaMemsetAsync(items[i].out_device, 0, (size_t)np * sizeof(float4),
                                            ctx->stream));
    }
    uint64_t launches = 0;
    Profile* prof = stats && ctx->prof.level > 0 ? &ctx->prof : nullptr;
    if (stats) {
        GBPT_CUDA_CHECK(cudaMemsetAsync(w.stats, 0, 4 * sizeof(unsigned long long), ctx->stream));
        GBPT_CUDA_CHECK(cudaMemsetAsync(ctx->d_misc, 0, 2 * sizeof(unsigned long long), ctx->stream));
        GBPT_CUDA_CHECK(cudaMemsetAsync(ctx->d_misc + 4, 0, 4 * sizeof(unsigned long long),
                                        ctx->stream));
        GBPT_CUDA_CHECK(cudaEventRecord(ctx->ev0, ctx->stream));
        if (prof) prof->reset();
    }
    ctx->batch.work = &w;
    ctx->batch.stream = ctx->stream;
    bool two = false;
    if ((rc = use_two_streams(ctx, prof, &two)) != GBPT_OK) return rc;
    if (two) {
        ctx->batch2.work = &ctx->work2;
        ctx->batch2.stream = ctx->stream2;
        ctx->batch2.use_graphs = ctx->batch.use_graphs;
        if (stats)
            GBPT_CUDA_CHECK(cudaMemsetAsync(ctx->work2.stats, 0, 4 * sizeof(unsigned long long),
                                            ctx->stream));
    }
    rc = render_batch(ctx->batch, items.data(), n, &launches, prof, ctx->d_misc,
                      two ? &ctx->batch2 : nullptr, ctx->ev_fork, ctx->ev_join);
    if (rc != GBPT_OK) {
        set_error(rc == GBPT_ERR_NO_MEMORY ? "gbpt_render_batch: work buffer allocation failed"
                                           : "gbpt_render_batch: launch failed: " +
                                                 cuda_error_string(cudaGetLastError()));
        return rc;
    }
    if (stats) GBPT_CUDA_CHECK(cudaEventRecord(ctx->ev1, ctx->stream));
    for (uint32_t i = 0; i < n; ++i) {
        if (!reqs[i].out_host) continue;
        GBPT_CUDA_CHECK(cudaMemcpyAsync(reqs[i].out_host, items[i].out_device,
                                        (size_t)items[i].pixel_count * sizeof(float4),
                                        cudaMemcpyDeviceToHost, ctx->stream));
    }
    if ((rc = check_device_error(ctx))) return rc;
    if (stats) return read_stats(ctx, samples, launches, prof, stats, two);
    return GBPT_OK;
}

GBPT_API int gbpt_set_graphs(gbpt_ctx* ctx, int enable) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->batch.use_graphs = enable != 0;
    ctx->batch2.use_graphs = enable != 0;
    ctx->tuning.use_graphs = enable != 0;
    if (!enable) {
        ctx->batch.release();
        ctx->batch2.release();
    }
    return GBPT_OK;
}

static int check_tuning(const gbpt_tuning* t) {
    if (!t || t->wave_paths > (1ull << 24) || (t->wave_paths && t->wave_paths < 1024) ||
        t->sort_materials < -1 || t->sort_materials > 1 || t->bvh_build < GBPT_BVH_SPLIT ||
        t->bvh_build > GBPT_BVH_MEDIUM || t->streams < 0 || t->streams > 2 ||
        t->trace_refill_lanes < 0 || t->trace_refill_lanes > 32 || t->trace_postpone_lanes < 0 ||
        t->trace_postpone_lanes > 32 || t->trace_blocks_per_sm < 0 ||
        t->trace_blocks_per_sm > 64) {
        set_error("tuning: wave_paths must be 0 or in [1024, 2^24], sort_materials in {-1, 0, 1}, "
                  "bvh_build a GBPT_BVH_* value, streams in {0, 1, 2}, trace_refill_lanes and "
                  "trace_postpone_lanes in [0, 32], trace_blocks_per_sm in [0, 64]");
        return GBPT_ERR_INVALID;
    }
    return GBPT_OK;
}


GBPT_API int gbpt_set_tuning(gbpt_ctx* ctx, const gbpt_tuning* t) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = check_tuning(t))) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->tuning = *t;
    ctx->batch.wave = t->wave_paths ? t->wave_paths : kWavePaths;
    ctx->batch.use_graphs = t->use_graphs != 0;
    ctx->batch.sched = sched_of(*t);
    ctx->batch.release();
    ctx->batch2.release();
    return GBPT_OK;
}

GBPT_API int gbpt_get_tuning(gbpt_ctx* ctx, gbpt_tuning* t) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!t) {
        set_error("gbpt_get_tuning: null output");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    *t = ctx->tuning;
    return GBPT_OK;
}

// The autotuner: candidate tunings rendered on one representative request, the fastest kept.
// Outputs do not depend on the tuning (tick size, shading order and warp scheduling only change
// the schedule), so only time is compared. Stage 1 crosses tick size and material sorting; the
// traversal's refill and postponement thresholds and its blocks per SM are then searched one at a
// time from the best so far. Results are cached per bucket of scene size, frame size, path length
// and estimator.
GBPT_API int gbpt_autotune(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                           const gbpt_render_params* p, gbpt_tuning* out, double* ms_out) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = validate_params(camera, p))) return rc;
    if (p->pixel_count) {
        set_error("gbpt_autotune: tune on a whole frame (no pixel list)");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_autotune: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    if (ms_out)
        for (int i = 0; i < GBPT_AUTOTUNE_CANDIDATES; ++i) ms_out[i] = std::nan("");
    const uint32_t n_pix = p->width * p->height;
    auto log2_bucket = [](uint64_t x) {
        int b = 0;
        while (x > 1) {
            x >>= 1;
            ++b;
        }
        return b;
    };
    const std::array<int, 5> key{log2_bucket(std::max<uint64_t>(it->second.n_tris, 1)),
                                 log2_bucket(std::max<uint64_t>((uint64_t)n_pix * p->spp, 1)),
                                 p->max_path_length, p->nee ? 1 : 0, p->rr_depth};
    auto apply = [&](const gbpt_tuning& t) {
        ctx->tuning = t;
        ctx->batch.wave = t.wave_paths;
        ctx->batch.sched = sched_of(t);
        ctx->batch.release();
        ctx->batch2.release();
        if (out) *out = t;
    };
    const auto cached = ctx->tune_cache.find(key);
    if (cached != ctx->tune_cache.end()) {
        gbpt_tuning t = cached->second.tuning;
        t.use_graphs = ctx->tuning.use_graphs;
        t.bvh_build = ctx->tuning.bvh_build;
        t.streams = ctx->tuning.streams;
        if (ms_out)
            for (int i = 0; i < GBPT_AUTOTUNE_CANDIDATES; ++i) ms_out[i] = cached->second.ms[i];
        apply(t);
        return GBPT_OK;
    }
    Work& w = ctx->work;
    if (n_pix > w.out_cap) {
        if (w.out) cudaFree(w.out);
        w.out = nullptr;
        w.out_cap = 0;
        GBPT_CUDA_CHECK(device_malloc((void**)&w.out, (size_t)n_pix * sizeof(float4)));
        w.out_cap = n_pix;
    }
    std::array<double, GBPT_AUTOTUNE_CANDIDATES> ms_all;
    ms_all.fill(std::nan(""));
    // one candidate: a warm-up render (it also allocates), then the timed one
    auto time_one = [&](const gbpt_tuning& t, int idx, double* ms_res) -> int {
        RenderArgs a;
        a.camera = *camera;
        a.params = *p;
        a.params.sort_materials = t.sort_materials;
        a.pixel_count = n_pix;
        a.pixels_device = nullptr;
        a.out_device = w.out;
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {
            GBPT_CUDA_CHECK(cudaEventRecord(ctx->ev0, ctx->stream));
            const int r = render_frame(it->second, w, a, ctx->stream, nullptr, nullptr, nullptr,
                                       t.wave_paths, nullptr, nullptr, nullptr, nullptr,
                                       sched_of(t));
            if (r != GBPT_OK) {
                set_error("gbpt_autotune: render failed");
                return r;
            }
            GBPT_CUDA_CHECK(cudaEventRecord(ctx->ev1, ctx->stream));
            GBPT_CUDA_CHECK(cudaEventSynchronize(ctx->ev1));
            GBPT_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        }
        ms_all[idx] = ms;
        *ms_res = ms;
        return GBPT_OK;
    };
    gbpt_tuning best = ctx->tuning;
    {
        const TraceSched defaults;
        best.trace_refill_lanes = (int32_t)defaults.refill_lanes;
        best.trace_postpone_lanes = (int32_t)defaults.postpone_lanes;
        best.trace_blocks_per_sm = 0; // every resident block
    }
    double best_ms = 1e300;
    auto consider = [&](const gbpt_tuning& t, int idx) -> int {
        double ms = 0.0;
        const int r = time_one(t, idx, &ms);
        if (r == GBPT_OK && ms < best_ms) {
            best_ms = ms;
            best = t;
        }
        return r;
    };
    // Tick sizes, largest first. A tick's wave bounds how many requests share it; on a frame that
    // fits every candidate wave the timings tie within noise, so a smaller wave is taken only when
    // it is at least 2 % faster (a served stream of small requests otherwise ran in 2^21-path
    // ticks: six times the ticks of 2^24, 12 % less throughput).
    const uint64_t waves[4] = {1ull << 21, 1ull << 22, 1ull << 23, 1ull << 24};
    for (int wi = 3; wi >= 0; --wi) {
        if (waves[wi] < (uint64_t)p->spp) continue;
        for (int sort = 0; sort < 2; ++sort) {
            gbpt_tuning t = best;
            t.wave_paths = waves[wi];
            t.sort_materials = sort;
            double ms = 0.0;
            if ((rc = time_one(t, 2 * wi + sort, &ms))) return rc;
            const bool smaller = best_ms < 1e300 && t.wave_paths < best.wave_paths;
            if (ms < (smaller ? 0.98 * best_ms : best_ms)) {
                best_ms = ms;
                best = t;
            }
        }
    }
    const int refill[5] = {12, 16, 20, 24, 28}, postpone[5] = {2, 4, 6, 8, 12};
    const int blocks[3] = {6, 7, 0};
    const gbpt_tuning stage1 = best;
    for (int k = 0; k < 5; ++k) {
        gbpt_tuning t = stage1;
        t.trace_refill_lanes = refill[k];
        if ((rc = consider(t, 8 + k))) return rc;
    }
    const gbpt_tuning stage2 = best;
    for (int k = 0; k < 5; ++k) {
        gbpt_tuning t = stage2;
        t.trace_postpone_lanes = postpone[k];
        if ((rc = consider(t, 13 + k))) return rc;
    }
    const gbpt_tuning stage3 = best;
    for (int k = 0; k < 3; ++k) {
        gbpt_tuning t = stage3;
        t.trace_blocks_per_sm = blocks[k];
        if ((rc = consider(t, 18 + k))) return rc;
    }
    if ((rc = check_device_error(ctx))) return rc;
    best.use_graphs = ctx->tuning.use_graphs;
    best.bvh_build = ctx->tuning.bvh_build;
    best.streams = ctx->tuning.streams;
    ctx->tune_cache[key] = gbpt_ctx::TuneResult{best, ms_all};
    if (ms_out)
        for (int i = 0; i < GBPT_AUTOTUNE_CANDIDATES; ++i) ms_out[i] = ms_all[i];
    apply(best);
    return GBPT_OK;
}

GBPT_API int gbpt_debug_primary_points(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                       const gbpt_render_params* p, float* out_host) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = validate_params(camera, p))) return rc;
    if (!out_host) {
        set_error("gbpt_debug_primary_points: null output");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_debug_primary_points: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    Work& w = ctx->work;
    const uint32_t n_pix = p->pixel_count ? p->pixel_count : p->width * p->height;
    RenderArgs a;
    a.camera = *camera;
    a.params = *p;
    a.pixel_count = n_pix;
    a.pixels_device = nullptr;
    a.out_device = nullptr;
    if (p->pixel_count) {
        if (p->pixel_count > w.pix_id_cap) {
            if (w.pix_id) cudaFree(w.pix_id);
            w.pix_id = nullptr;
            w.pix_id_cap = 0;
            GBPT_CUDA_CHECK(device_malloc((void**)&w.pix_id, (size_t)p->pixel_count * 4));
            w.pix_id_cap = p->pixel_count;
        }
        GBPT_CUDA_CHECK(cudaMemcpyAsync(w.pix_id, p->pixels, (size_t)p->pixel_count * 4,
                                        cudaMemcpyHostToDevice, ctx->stream));
        a.pixels_device = w.pix_id;
    }
    float* d = nullptr;
    const size_t bytes = (size_t)n_pix * 24 * sizeof(float);
    GBPT_CUDA_CHECK(device_malloc((void**)&d, bytes));
    rc = primary_points(it->second, w, a, ctx->stream, d);
    if (rc == GBPT_OK) {
        const cudaError_t e = cudaMemcpyAsync(out_host, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = GBPT_ERR_CUDA;
    }
    cudaFree(d);
    if (rc != GBPT_OK) {
        set_error("gbpt_debug_primary_points failed");
        return rc;
    }
    return check_device_error(ctx);
}

GBPT_API int gbpt_trace_primary(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                                uint32_t width, uint32_t height, uint32_t instance_mask,
                                gbpt_hit* out_hits_host) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!camera || !out_hits_host || width == 0 || height == 0 ||
        (uint64_t)width * height > (1ull << 28)) {
        set_error("gbpt_trace_primary: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_trace_primary: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    const uint64_t n = (uint64_t)width * height;
    if (n > ctx->hits_cap) {
        if (ctx->d_hits) cudaFree(ctx->d_hits);
        ctx->d_hits = nullptr;
        ctx->hits_cap = 0;
        GBPT_CUDA_CHECK(device_malloc((void**)&ctx->d_hits, n * sizeof(gbpt_hit)));
        ctx->hits_cap = n;
    }
    rc = trace_primary(it->second, *camera, width, height, instance_mask, ctx->d_hits,
                       reinterpret_cast<uint32_t*>(ctx->d_misc + 2), ctx->stream);
    if (rc) {
        set_error("gbpt_trace_primary: launch failed");
        return rc;
    }
    GBPT_CUDA_CHECK(cudaMemcpyAsync(out_hits_host, ctx->d_hits, n * sizeof(gbpt_hit),
                                    cudaMemcpyDeviceToHost, ctx->stream));
    return check_device_error(ctx);
}

GBPT_API int gbpt_gbuffer(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                          uint32_t width, uint32_t height, uint32_t instance_mask,
                          gbpt_gbuffer_texel* out_device) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!camera || !out_device || width == 0 || height == 0 ||
        (uint64_t)width * height > (1ull << 31)) {
        set_error("gbpt_gbuffer: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_gbuffer: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    rc = gbuffer(it->second, *camera, width, height, instance_mask, out_device,
                 reinterpret_cast<uint32_t*>(ctx->d_misc + 2), ctx->stream);
    if (rc) set_error("gbpt_gbuffer: launch failed");
    return rc;
}

static int trace_common(gbpt_ctx* ctx, uint32_t scene, const gbpt_ray* rays, uint32_t n,
                        uint32_t mask, int any_hit, gbpt_hit* hits, double* npr, double* tpr) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((n && (!rays || !hits))) {
        set_error("gbpt_trace: null rays or hits");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_trace: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    if (npr || tpr) GBPT_CUDA_CHECK(cudaMemsetAsync(ctx->d_misc, 0, 2 * sizeof(unsigned long long), ctx->stream));
    rc = trace_rays(it->second, rays, n, mask, any_hit, hits, ctx->d_misc, ctx->stream,
                    sched_of(ctx->tuning));
    if (rc) {
        set_error("gbpt_trace: launch failed");
        return rc;
    }
    if (npr || tpr) {
        unsigned long long c[2] = {0, 0};
        GBPT_CUDA_CHECK(cudaMemcpyAsync(c, ctx->d_misc, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
        if ((rc = check_device_error(ctx))) return rc;
        if (npr) *npr = n ? (double)c[0] / n : 0.0;
        if (tpr) *tpr = n ? (double)c[1] / n : 0.0;
    }
    return GBPT_OK;
}

GBPT_API int gbpt_trace(gbpt_ctx* ctx, uint32_t scene, const gbpt_ray* rays_device, uint32_t n,
                        uint32_t instance_mask, int any_hit, gbpt_hit* hits_device) {
    return trace_common(ctx, scene, rays_device, n, instance_mask, any_hit, hits_device, nullptr,
                        nullptr);
}

GBPT_API int gbpt_trace_counted(gbpt_ctx* ctx, uint32_t scene, const gbpt_ray* rays_device,
                                uint32_t n, uint32_t instance_mask, int any_hit,
                                gbpt_hit* hits_device, double* nodes_per_ray,
                                double* tris_per_ray) {
    double a = 0, b = 0;
    const int rc = trace_common(ctx, scene, rays_device, n, instance_mask, any_hit, hits_device, &a, &b);
    if (nodes_per_ray) *nodes_per_ray = a;
    if (tris_per_ray) *tris_per_ray = b;
    return rc;
}

// Camera::recompute_ray_basis + Camera::write_to (camera.cpp:263-266,349-367), focus on target
GBPT_API int gbpt_camera_look_at(const float position[3], const float target[3], const float up[3],
                                 float vfov, float aspect, float near_plane, float far_plane,
                                 gbpt_camera* out) {
    if (!position || !target || !up || !out) {
        set_error("gbpt_camera_look_at: null argument");
        return GBPT_ERR_INVALID;
    }
    const V3 pos = v3(position[0], position[1], position[2]);
    const V3 tgt = v3(target[0], target[1], target[2]);
    const V3 upv = v3(up[0], up[1], up[2]);
    const V3 fwd = normalize(tgt - pos);
    const V3 rgt = normalize(cross(fwd, upv));
    const V3 d = tgt - pos;
    const float focus = std::sqrt(dot(d, d));
    const float ht = std::tan(vfov * 0.5f);
    const V3 U = (ht * aspect * focus) * rgt;
    const V3 V = (ht * focus) * cross(rgt, fwd);
    const V3 W = focus * fwd;
    std::memset(out, 0, sizeof(*out));
    const float* src[4] = {&pos.x, &U.x, &V.x, &W.x};
    float* dst[4] = {out->position, out->U, out->V, out->W};
    for (int k = 0; k < 4; ++k) {
        dst[k][0] = src[k][0];
        dst[k][1] = src[k][1];
        dst[k][2] = src[k][2];
    }
    out->near_plane = near_plane;
    out->far_plane = far_plane;
    return GBPT_OK;
}

GBPT_API uint32_t gbpt_encode_normal(const float n[3]) { return encode_normal(v3(n[0], n[1], n[2])); }

GBPT_API uint32_t gbpt_pack_half2(float x, float y) { return pack_half2(x, y); }

} // extern "C"

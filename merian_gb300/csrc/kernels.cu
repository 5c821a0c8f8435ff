// Ray queries outside the wavefront (the caller's rays and the primary-hit buffer), and rendering
// from the library's fixed scratch array.
//
// The wavefront engine itself (request tables, ticks and their kernels) is wavefront.cu.
#include "device_shading.cuh"

#include <algorithm>
#include <cstdio>
#include <type_traits>

namespace gbpt {

std::string cuda_error_string(cudaError_t e) { return std::string(cudaGetErrorString(e)); }

namespace {

// merian's Hit (hit.slang:25-65): for two-level hits the custom index of the instance (the first
// geometry of its BLAS), the TLAS instance and the geometry within the BLAS; misses all ~0.
GBPT_DI gbpt_hit to_hit(const DevScene& sc, const Hit& h) {
    gbpt_hit out;
    const bool ok = h.geom != kNoInst;
    uint32_t first = 0;
    if (ok && h.inst != kNoInst) first = __float_as_uint(__ldg(&sc.inst[7ull * h.inst + 6]).z);
    out.instance_id = ok ? first : kNoInst;
    out.instance_index = ok ? (h.inst == kNoInst ? 0u : h.inst) : kNoInst;
    out.primitive_id = h.prim;
    out.geometry_index = ok ? h.geom - first : kNoInst;
    out.barycentrics[0] = ok ? h.u : 0.f;
    out.barycentrics[1] = ok ? h.v : 0.f;
    out.t = ok ? h.t : -1.0f;
    out.reserved = 0;
    return out;
}

// The caller's rays through the persistent traversal (the closest hit or, with ANY, any hit).
template <bool ANY>
__global__ void __launch_bounds__(128, kTraceBlocksPerSM)
    k_trace_rays(DevScene sc, const gbpt_ray* rays, uint32_t n, uint32_t mask, gbpt_hit* hits,
                 unsigned long long* work_ctr, uint32_t* fetch, uint32_t* err, int refill_lanes,
                 int postpone_lanes) {
    TraceCounters ctr{0, 0, 0, 0, 0, 0};
    auto load = [&](uint32_t i, TraceState& s) {
        const gbpt_ray r = rays[i];
        s.nodes = sc.nodes;
        s.tris_base = sc.tris;
        s.tri_stride = sc.tri_stride;
        s.insts = sc.n_inst ? sc.inst : nullptr;
        s.mask = mask;
        trace_init(s, f3(r.origin[0], r.origin[1], r.origin[2]),
                   f3(r.direction[0], r.direction[1], r.direction[2]), r.tmin, r.tmax);
    };
    auto store = [&](uint32_t i, const Hit& h) { hits[i] = to_hit(sc, h); };
    auto alpha = [&](uint32_t, uint32_t g, uint32_t p, float u, float v) {
        return alpha_discard(sc, g, p, u, v);
    };
    trace_persistent<ANY, true, true>(n, fetch, load, store, alpha, &ctr, err, refill_lanes,
                                      postpone_lanes);
    if (work_ctr) {
        atomicAdd(work_ctr + 0, (unsigned long long)ctr.nodes);
        atomicAdd(work_ctr + 1, (unsigned long long)ctr.tris);
    }
}

// The primary hit of every pixel (the GBuffer's visibility pass, gbuffer_rt.slang:18-58).
__global__ void k_trace_primary(DevScene sc, CamGPU cam, uint32_t w, uint32_t h, uint32_t mask,
                                gbpt_hit* hits, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    float3 o, d;
    float tmin, tmax;
    camera_ray(cam, i % w, i / w, w, h, o, d, tmin, tmax);
    hits[i] = to_hit(sc, trace_ray<false, false>(sc, o, d, tmin, tmax, mask, nullptr, err));
}

GBPT_DI uint32_t pack_half2_rn(float lo, float hi) {
    return (uint32_t)__half_as_ushort(__float2half_rn(lo)) |
           ((uint32_t)__half_as_ushort(__float2half_rn(hi)) << 16);
}

// camera.slang:34-37 for a pixel of the frame
GBPT_DI float3 pinhole_direction(const CamGPU& c, uint32_t px, uint32_t py, uint32_t w,
                                 uint32_t h) {
    const float x = (((float)px + 0.5f) + c.jx) / (float)w;
    const float y = (((float)py + 0.5f) + c.jy) / (float)h;
    return normalize((2.0f * x - 1.0f) * c.U + (-2.0f * y + 1.0f) * c.V + c.W);
}

// The GBuffer (Raytraced) node for a static camera (gbuffer_rt.slang:18-94): hit, shading
// normal, depth and its screen gradient, albedo and emission per pixel. Motion vectors are 0 and
// delta_z is |pos - camera| - linear_z: the previous camera and transforms equal the current ones.
__global__ void k_gbuffer(DevScene sc, CamGPU cam, uint32_t w, uint32_t h, uint32_t mask,
                          gbpt_gbuffer_texel* out, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const uint32_t px = i % w, py = i / w;
    float3 o, d;
    float tmin, tmax;
    camera_ray(cam, px, py, w, h, o, d, tmin, tmax);
    const Hit ht = trace_ray<false, false>(sc, o, d, tmin, tmax, mask, nullptr, err);
    gbpt_gbuffer_texel t;
    const bool hit = ht.geom != 0xFFFFFFFFu;
    const gbpt_hit ph = to_hit(sc, ht);
    t.instance_id = ph.instance_id;
    t.primitive_id = ph.primitive_id;
    t.geometry_index = (uint16_t)ph.geometry_index;
    t.instance_index = (uint16_t)ph.instance_index;
    t.barycentrics = hit ? pack_half2_rn(ht.u, ht.v) : 0u;
    t.motion[0] = t.motion[1] = 0.0f;
    t.grad_z = 0u;
    t.delta_z = 0.0f;
    SPd sp;
    if (!hit || ht.geom >= sc.geom_count) sp = env_sp(sc, o, d);
    else sp = surface_sp(sc, o, d, ht.geom, ht.prim, ht.u, ht.v, ht.inst);
    const float lz = length(sp.pos - o);
    t.linear_z = fminf(lz, 65504.0f);
    t.encoded_normal = encode_normal(sp.frame.n);
    float3 albedo = sp.emission;
    if (!sp.env) {
        // Surface::compute_grad_z (hit.slang:99-103)
        const float n_dot_oo = dot(sp.fn, sp.pos - o);
        const float gx = n_dot_oo / dot(sp.fn, pinhole_direction(cam, px + 1, py, w, h)) - lz;
        const float gy = n_dot_oo / dot(sp.fn, pinhole_direction(cam, px, py + 1, w, h)) - lz;
        t.grad_z = pack_half2_rn(gx, gy);
        t.delta_z = length(sp.pos - cam.pos) - lz;
        const Material m = load_material(sc, sp.mat, sp.front, 1.0f, sp.tex_color);
        albedo = material_albedo(m, sp.frame.to_local(-d));
    }
    t.albedo[0] = albedo.x;
    t.albedo[1] = albedo.y;
    t.albedo[2] = albedo.z;
    t.emission[0] = sp.emission.x;
    t.emission[1] = sp.emission.y;
    t.emission[2] = sp.emission.z;
    out[i] = t;
}

CamGPU to_cam(const gbpt_camera& c) {
    CamGPU g;
    g.pos = make_float3(c.position[0], c.position[1], c.position[2]);
    g.U = make_float3(c.U[0], c.U[1], c.U[2]);
    g.V = make_float3(c.V[0], c.V[1], c.V[2]);
    g.W = make_float3(c.W[0], c.W[1], c.W[2]);
    g.near_plane = c.near_plane;
    g.far_plane = c.far_plane;
    g.jx = c.jitter[0];
    g.jy = c.jitter[1];
    return g;
}

} // namespace

int trace_rays(const SceneGPU& scene, const gbpt_ray* rays, uint32_t n, uint32_t mask, int any_hit,
               gbpt_hit* hits, unsigned long long* work_ctr, cudaStream_t st,
               const TraceSched& sched) {
    if (n == 0) return GBPT_OK;
    const DevScene sc = make_dev_scene(scene);
    uint32_t* err = reinterpret_cast<uint32_t*>(work_ctr + 2);
    uint32_t* fetch = reinterpret_cast<uint32_t*>(work_ctr + 3);
    cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st);
    const int cap = sched.blocks_per_sm ? (int)sched.blocks_per_sm * num_sms() : 1 << 30;
    const int ra = (int)sched.refill_lanes, po = (int)sched.postpone_lanes;
    if (any_hit)
        k_trace_rays<true><<<std::min(persistent_grid(k_trace_rays<true>), cap), 128, 0, st>>>(
            sc, rays, n, mask & 0xFFu, hits, work_ctr, fetch, err, ra, po);
    else
        k_trace_rays<false><<<std::min(persistent_grid(k_trace_rays<false>), cap), 128, 0, st>>>(
            sc, rays, n, mask & 0xFFu, hits, work_ctr, fetch, err, ra, po);
    return cudaGetLastError() == cudaSuccess ? GBPT_OK : GBPT_ERR_CUDA;
}

int gbuffer(const SceneGPU& scene, const gbpt_camera& cam, uint32_t w, uint32_t h, uint32_t mask,
            gbpt_gbuffer_texel* out, uint32_t* err, cudaStream_t st) {
    const DevScene sc = make_dev_scene(scene);
    const uint32_t n = w * h;
    k_gbuffer<<<(n + 127) / 128, 128, 0, st>>>(sc, to_cam(cam), w, h, mask & 0xFFu, out, err);
    return cudaGetLastError() == cudaSuccess ? GBPT_OK : GBPT_ERR_CUDA;
}

int trace_primary(const SceneGPU& scene, const gbpt_camera& cam, uint32_t w, uint32_t h,
                  uint32_t mask, gbpt_hit* hits, uint32_t* err, cudaStream_t st) {
    const DevScene sc = make_dev_scene(scene);
    const uint32_t n = w * h;
    k_trace_primary<<<(n + 127) / 128, 128, 0, st>>>(sc, to_cam(cam), w, h, mask & 0xFFu, hits, err);
    return cudaGetLastError() == cudaSuccess ? GBPT_OK : GBPT_ERR_CUDA;
}

// ---- rendering without allocation ------------------------------------------------------------------
// Some callers must not allocate device memory while they render: a host whose allocator has
// already reserved the GPU for itself, a real-time loop that may not block in cudaMalloc/cudaFree
// (both can synchronise the device), or a process under a hard memory budget fixed at start-up.
// For them the same wavefront runs with every scratch buffer carved from this fixed array, which
// each GPU that loads the library holds until the process exits. Every call shares it and it keeps
// the last call's contents: the counters are cleared per call, and calls that overlap on the GPU
// (other streams, other host threads) race on it.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {
constexpr uint64_t kStaticCounterBytes = 256; // 16 counters + 8 stats words, padded
constexpr uint64_t kStaticPixelBytes = (uint64_t)kStaticMaxPixelList * 4;
// per path: throughput and radiance (32), two ray queues (2 x 32), hits (32), shadow queue (52);
// plus a 112-byte primary point per pixel, budgeted as one pixel per path
constexpr uint64_t kStaticBytesPerPath = 32 + 2 * 32 + 32 + (32 + 16 + 4) + 16 * kPixFloat4;
// alignment padding of the carved arrays, and the tick tables of a one-request render
constexpr uint64_t kStaticSlackBytes = 16 * 256 + 1024;

// The array's device address on the current device. Host code cannot use the symbol itself (it
// names a host-side stand-in), so every call asks the runtime: the lookup allocates nothing, and
// an address cached across calls would dangle after a device reset reloads the module. The first
// lookup on a device may load the module, which is why the first call belongs before any capture.
int static_scratch_address(unsigned char** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) return GBPT_ERR_CUDA;
    *out = (unsigned char*)p;
    return GBPT_OK;
}
} // namespace

uint64_t static_scratch_paths() {
    // kStaticSlackBytes for the alignment of the carved arrays and the tick tables
    return (kStaticScratchBytes - kStaticCounterBytes - kStaticPixelBytes - kStaticSlackBytes) /
           kStaticBytesPerPath;
}

int render_frame_static(const SceneGPU& scene, const RenderArgs& args, const uint32_t* pixels_host,
                        cudaStream_t st, std::string& err) {
    unsigned char* base = nullptr;
    int rc = static_scratch_address(&base);
    if (rc != GBPT_OK) {
        err = "cudaGetSymbolAddress of the static scratch array failed";
        return rc;
    }
    const uint64_t N = static_scratch_paths();
    const uint64_t S = (uint64_t)args.params.spp;
    if (S > N) {
        err = "spp " + std::to_string(S) + " exceeds the " + std::to_string(N) +
              " paths the static scratch holds per wave";
        return GBPT_ERR_INVALID;
    }
    if (args.pixel_count > kStaticMaxPixelList && pixels_host) {
        err = "pixel list longer than " + std::to_string(kStaticMaxPixelList) + " entries";
        return GBPT_ERR_INVALID;
    }
    // carve the work buffers: counters, pixel list, per-path and per-pixel arrays, then the
    // request tables in what is left
    Work w;
    w.fixed = true;
    w.path_cap = N;
    w.pixel_cap = N;
    unsigned char* p = base;
    w.counters = (uint32_t*)p;
    w.stats = (unsigned long long*)(p + 64);
    p += kStaticCounterBytes;
    uint32_t* pix_ids = (uint32_t*)p;
    p += kStaticPixelBytes;
    auto carve = [&](auto*& ptr, uint64_t count) {
        using T = std::remove_reference_t<decltype(*ptr)>;
        ptr = (T*)p;
        p += (count * sizeof(T) + 255) & ~255ull;
    };
    carve(w.path, 2 * N);
    carve(w.q_od[0], 2 * N);
    carve(w.q_od[1], 2 * N);
    carve(w.hit, 2 * N);
    carve(w.s_od, 2 * N);
    carve(w.s_contrib, N);
    carve(w.s_path, N);
    carve(w.pix, kPixFloat4 * N);
    const uint64_t used = (uint64_t)(p - base);
    if (used + tick_table_bytes(1) > kStaticScratchBytes) {
        err = "static scratch layout overflow";
        return GBPT_ERR_INVALID;
    }
    w.tables = p;
    w.tables_bytes = kStaticScratchBytes - used;
    if (cudaMemsetAsync(w.counters, 0, kStaticCounterBytes, st) != cudaSuccess) {
        err = "cudaMemsetAsync failed";
        return GBPT_ERR_CUDA;
    }
    RenderArgs a = args;
    if (pixels_host && args.pixel_count) {
        if (cudaMemcpyAsync(pix_ids, pixels_host, (size_t)args.pixel_count * 4,
                            cudaMemcpyHostToDevice, st) != cudaSuccess) {
            err = "cudaMemcpyAsync of the pixel list failed";
            return GBPT_ERR_CUDA;
        }
        a.pixels_device = pix_ids;
    } else {
        a.pixels_device = nullptr;
    }
    rc = render_frame(scene, w, a, st, nullptr, nullptr, nullptr);
    if (rc != GBPT_OK) {
        err = "render launch failed";
        return rc;
    }
    uint32_t flag = 0;
    if (cudaMemcpyAsync(&flag, w.counters + 3, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        err = "synchronisation failed";
        return GBPT_ERR_CUDA;
    }
    if (flag) {
        err = "kernel error flag raised (traversal stack overflow)";
        return GBPT_ERR_DEVICE;
    }
    return GBPT_OK;
}

} // namespace gbpt

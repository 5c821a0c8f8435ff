// The wavefront engine: one or many render requests advanced in ticks.
//
// merian renders one request per dispatch, one ray-generation thread per pixel looping over
// samples and bounces (render_pt.slang:92-130, trace_path :24-90). Here every request (scene,
// camera, spp, path length, estimator, output) is split into chunks of whole pixels, and a tick
// packs chunks of any number of requests into one wave of at most kWavePaths (pixel, sample)
// paths. A tick is a fixed kernel sequence on one stream:
//   k_primary        camera ray, closest hit, primary shading point per pixel (the GBuffer hit,
//                    barycentrics rounded to half as the GBuffer stores them, gbuffer.slang:40-60)
//   k_shade_primary  per path: RNG pcg4d16(pixel, frame, sample), emission on primary, scatter
//   k = 2..L:        k_trace (closest hit of the ray queue) -> k_shade (emission with MIS,
//                    roulette, NEE, BSDF sample, ray append) -> k_shadow (any hit of NEE rays)
//   k_finalize       per pixel: samples summed in a fixed order, NaN/Inf dropped but counted
// Queue entries carry (chunk << 24 | path), so rays of different scenes share one launch; a
// chunk holds its scene's traversal pointers. Each pixel's samples live in one tick and are summed
// in a fixed order, so a request's result is bit-identical alone and in any mix of requests.
#include "device_shading.cuh"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

namespace gbpt {

namespace {

// queue entry = chunk << 24 | path: waves of up to 2^24 paths (the largest spp a request may
// ask for), up to 256 chunks per tick
constexpr uint32_t kPathBits = 24;
constexpr uint32_t kPathMask = (1u << kPathBits) - 1u;
constexpr uint32_t kMaxChunks = 256;
constexpr uint64_t kMaxWavePaths = 1ull << kPathBits;
static_assert(kWavePaths <= kMaxWavePaths, "path ids must fit the packed queue entry");

// resident 128-thread blocks per SM the shading kernels are register-budgeted for
// (65536 / (5 * 128) = 102 registers per thread)
#ifndef GBPT_SHADE_BLOCKS_PER_SM
#define GBPT_SHADE_BLOCKS_PER_SM 5
#endif
constexpr int kShadeBlocksPerSM = GBPT_SHADE_BLOCKS_PER_SM;
// the primary-hit kernel's budget (it traces one camera ray per thread, then shades the hit):
// 64 registers and some spills beat the 164 registers it takes unbounded (3 blocks per SM) on
// the 640x360 frame (primary + finalize 0.58 against 0.68 ms; 4 / 6 / 10 / 12 blocks: 0.65 /
// 0.63 / 0.64 / 0.57)
#ifndef GBPT_PRIMARY_BLOCKS_PER_SM
#define GBPT_PRIMARY_BLOCKS_PER_SM 8
#endif
constexpr int kPrimaryBlocksPerSM = GBPT_PRIMARY_BLOCKS_PER_SM;

constexpr uint32_t kReqEmission = 1u, kReqNee = 2u, kReqDemodulate = 4u;

// "shader execution reordering" (render_pt.cpp:160-161): the closest-hit queue is ordered by
// material model before shading, so the warps of k_shade run one BSDF model at a time. Keys:
// 0 environment (miss or UseEnvMap geometry), 1 diffuse, 2 OpenPBR, 3 OpenPBR with transmission.
// Shading results do not depend on the order (each entry updates only its own path).
constexpr int kSortKeys = 4;

struct ReqGPU {
    CamGPU cam;
    uint32_t width, height, spp, max_len;
    uint32_t flags, mask, frame;
    int32_t rr_depth;
    uint32_t scene;
    uint32_t pad;
    const uint32_t* pixels; // device list or nullptr
    float4* out;            // device output, indexed by list index
};

struct ChunkGPU {
    uint32_t req;       // request index
    uint32_t scene;     // scene table index
    uint32_t pix_first; // first list index of the chunk's pixels
    uint32_t n_pix;
    uint32_t slot_base; // first pixel slot of the tick
    uint32_t path_base; // first path of the tick
    uint32_t spp;
    uint32_t mask;
    const uint4* nodes; // the scene's traversal data, for the trace kernels
    const float4* tris;
    const float4* insts; // instance records of a two-level scene, else nullptr
    const uint8_t* geom_key; // material-sort key of each geometry of the scene
    uint32_t tri_stride;     // float4 from one copy of the triangle records to the next
    uint32_t pad2;
};
static_assert(sizeof(ChunkGPU) == 72, "chunk layout");

struct TickHeader {
    uint32_t n_chunks, n_pix, n_paths, pad;
};

struct TickArgs {
    const DevScene* scenes;
    const ReqGPU* reqs;
    const ChunkGPU* chunks;
    const TickHeader* hdr;
    Work w;
    int refill_lanes, postpone_lanes; // warp scheduling of the persistent traversal
};

// last chunk whose base <= key
GBPT_DI uint32_t chunk_by_slot(const ChunkGPU* c, uint32_t n, uint32_t q) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (c[mid].slot_base <= q) lo = mid;
        else hi = mid;
    }
    return lo;
}
GBPT_DI uint32_t chunk_by_path(const ChunkGPU* c, uint32_t n, uint32_t p) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (c[mid].path_base <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

GBPT_DI uint32_t pixel_id(const ReqGPU& r, uint32_t li) { return r.pixels ? __ldg(&r.pixels[li]) : li; }

// Primary hit + shading point per pixel slot (gbuffer_rt.slang:18-58, render_pt.slang:98-103)
__global__ void __launch_bounds__(128, kPrimaryBlocksPerSM) k_primary(TickArgs t, int sort) {
    const uint32_t n = t.hdr->n_pix, nc = t.hdr->n_chunks;
    const uint32_t stride = gridDim.x * blockDim.x;
    // with material-sorted shading: the key of each pixel's primary hit for all its paths
    __shared__ uint32_t key_count[kSortKeys];
    if (threadIdx.x < kSortKeys) key_count[threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        const ChunkGPU c = t.chunks[chunk_by_slot(t.chunks, nc, q)];
        const ReqGPU& r = t.reqs[c.req];
        const DevScene& sc = t.scenes[c.scene];
        const uint32_t pid = pixel_id(r, c.pix_first + (q - c.slot_base));
        const uint32_t px = pid % r.width, py = pid / r.width;
        float3 o, d;
        float tmin, tmax;
        camera_ray(r.cam, px, py, r.width, r.height, o, d, tmin, tmax);
        const Hit h = trace_ray<false, false>(sc, o, d, tmin, tmax, c.mask, nullptr,
                                              t.w.counters + 3);
        if (sort) {
            const uint32_t key = h.geom < sc.geom_count ? __ldg(&c.geom_key[h.geom]) : 0u;
            uint8_t* kp = t.w.keys + c.path_base + (q - c.slot_base) * c.spp;
            for (uint32_t s2 = 0; s2 < c.spp; ++s2) kp[s2] = (uint8_t)key;
            atomicAdd(&key_count[key], c.spp);
        }
        SPd sp;
        if (h.geom == 0xFFFFFFFFu || h.geom >= sc.geom_count) {
            sp = env_sp(sc, o, d);
        } else {
            sp = surface_sp(sc, o, d, h.geom, h.prim, round_half(h.u), round_half(h.v), h.inst);
        }
        float4* pc = t.w.pix + kPixFloat4 * q;
        pc[0] = make_float4(sp.pos.x, sp.pos.y, sp.pos.z, __uint_as_float(sp.enc_fn));
        pc[1] = make_float4(sp.frame.n.x, sp.frame.n.y, sp.frame.n.z, __uint_as_float(sp.mat));
        const uint32_t fl = (sp.has_material ? 1u : 0u) | (sp.front ? 2u : 0u);
        pc[2] = make_float4(sp.frame.t.x, sp.frame.t.y, sp.frame.t.z, __uint_as_float(fl));
        // "demodulate albedo": the GBuffer's albedo, floored at 1e-2 (gbuffer.slang:135-140),
        // from the full-precision hit as the GBuffer node computes it (gbuffer_rt.slang:67-69)
        float3 demod = f3(1.f, 1.f, 1.f);
        if (r.flags & kReqDemodulate) {
            float3 a = sp.emission;
            if (!sp.env) {
                const SPd ex = surface_sp(sc, o, d, h.geom, h.prim, h.u, h.v, h.inst);
                a = ex.env ? ex.emission
                           : material_albedo(load_material(sc, ex.mat, ex.front, 1.0f,
                                                           ex.tex_color),
                                             ex.frame.to_local(-d));
            }
            demod = f3(fmaxf(a.x, 1e-2f), fmaxf(a.y, 1e-2f), fmaxf(a.z, 1e-2f));
        }
        pc[3] = make_float4(sp.frame.b.x, sp.frame.b.y, sp.frame.b.z, demod.x);
        pc[4] = make_float4(sp.emission.x, sp.emission.y, sp.emission.z, demod.y);
        pc[5] = make_float4(d.x, d.y, d.z, demod.z);
        pc[6] = make_float4(sp.tex_color.x, sp.tex_color.y, sp.tex_color.z, 0.f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(t.w.stats + 0, (unsigned long long)n);
    if (sort) {
        __syncthreads();
        if (threadIdx.x < kSortKeys && key_count[threadIdx.x])
            atomicAdd(t.w.counters + 8 + threadIdx.x, key_count[threadIdx.x]);
    }
}

// One iteration of the trace_path loop (render_pt.slang:35-79) from shading point sp, reached
// by `k` segments. Returns true and the next ray when the path continues; may emit a shadow ray.
// The estimator is a per-request flag, not a template parameter: every request runs the same
// machine code whatever else shares its tick, so the compiler's FMA contraction (and with it
// every rounding) is the same alone and in a batch.
GBPT_DI bool scatter(const DevScene& sc, const ReqGPU& r, int k, const SPd& sp, float3 ray_d,
                     float3& thr, float& ior, float& last_pdf, Pcg& rng, float3& no, float3& nd,
                     bool& want_shadow, float4& s_o, float4& s_d, float4& s_c) {
    want_shadow = false;
    if (!sp.has_material ||
        (thr.x < kThroughputMin && thr.y < kThroughputMin && thr.z < kThroughputMin))
        return false;
    if (r.rr_depth > 0 && k >= r.rr_depth) {
        const float q = fminf(1.0f, max3(thr));
        if (rng.next_float() >= q) return false;
        thr = thr / q;
    }
    const Material m = load_material(sc, sp.mat, sp.front, ior, sp.tex_color);
    const float3 wi_local = sp.frame.to_local(-ray_d);
    const float3 ng = decode_normal(sp.enc_fn);
    const float wi_ng = dot(-ray_d, ng);
    if (r.flags & kReqNee) {
        const LightSample ls = sample_light(sc, sp.pos, rng);
        if (ls.valid) {
            const float3 wl = sp.frame.to_local(ls.dir);
            const bool trans = wi_local.z * wl.z < 0.f;
            const float wl_ng = dot(ls.dir, ng);
            if (((wi_ng < 0.f) != (wl_ng < 0.f)) == trans) {
                const float3 f = material_eval(m, wi_local, wl);
                if (f.x > 0.f || f.y > 0.f || f.z > 0.f) {
                    const float pb = material_pdf(m, wi_local, wl);
                    const float wmis = power_heuristic(ls.pdf, pb);
                    const float3 c = thr * f * ls.le * (wmis / ls.pdf);
                    const float3 so = offset_ray_origin(sp.pos, wl_ng < 0.f ? -ng : ng);
                    s_o = make_float4(so.x, so.y, so.z, ls.dist);
                    s_d = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, 0.f);
                    s_c = make_float4(c.x, c.y, c.z, 0.f);
                    want_shadow = true;
                }
            }
        }
    }
    const BsdfSample bs = material_sample(m, wi_local, rng);
    if (!bs.valid) return false;
    const float3 wo = sp.frame.to_world(bs.wo);
    thr = thr * bs.weight;
    const bool transmission = wi_local.z * bs.wo.z < 0.f;
    if (transmission) ior = ior / m.eta;
    const float wo_ng = dot(wo, ng);
    if (((wi_ng < 0.f) != (wo_ng < 0.f)) != transmission) return false;
    no = offset_ray_origin(sp.pos, wo_ng < 0.f ? -ng : ng);
    nd = wo;
    last_pdf = bs.pdf;
    return true;
}

// Path start at the primary shading point (render_pt.slang:113-117) and the first scatter.
__global__ void __launch_bounds__(128, kShadeBlocksPerSM)
    k_shade_primary(TickArgs t, const uint32_t* __restrict__ perm) {
    const uint32_t n = t.hdr->n_paths, nc = t.hdr->n_chunks;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_round = (n + 31u) & ~31u;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_round; j += stride) {
        bool want = false, want_shadow = false;
        float3 no, nd;
        float4 s_o, s_d, s_c;
        uint32_t ci = 0, rng_state = 0;
        const uint32_t p = (perm && j < n) ? __ldg(&perm[j]) : j;
        if (j < n) {
            ci = chunk_by_path(t.chunks, nc, p);
            const ChunkGPU c = t.chunks[ci];
            const ReqGPU& r = t.reqs[c.req];
            const DevScene& sc = t.scenes[c.scene];
            const uint32_t local = p - c.path_base;
            const uint32_t slot = c.slot_base + local / c.spp, s = local % c.spp;
            const uint32_t pid = pixel_id(r, c.pix_first + local / c.spp);
            const uint32_t px = pid % r.width, py = pid / r.width;
            Pcg rng{pcg4d16(px, py, r.frame, s)};
            const float4* pc = t.w.pix + kPixFloat4 * slot;
            const float4 c0 = pc[0], c1 = pc[1], c2 = pc[2], c3 = pc[3], c4 = pc[4], c5 = pc[5];
            const float4 c6 = pc[6];
            SPd sp;
            sp.pos = f3(c0.x, c0.y, c0.z);
            sp.enc_fn = __float_as_uint(c0.w);
            sp.frame.n = f3(c1.x, c1.y, c1.z);
            sp.mat = __float_as_uint(c1.w);
            sp.frame.t = f3(c2.x, c2.y, c2.z);
            const uint32_t fl = __float_as_uint(c2.w);
            sp.has_material = (fl & 1u) != 0u;
            sp.front = (fl & 2u) != 0u;
            sp.frame.b = f3(c3.x, c3.y, c3.z);
            sp.emission = f3(c4.x, c4.y, c4.z);
            sp.tex_color = f3(c6.x, c6.y, c6.z);
            const float3 d = f3(c5.x, c5.y, c5.z);
            float3 thr = f3(1.f, 1.f, 1.f);
            float ior = 1.0f, last_pdf = 0.f;
            const float3 rad = (r.flags & kReqEmission) ? sp.emission : f3(0.f, 0.f, 0.f);
            if (r.max_len > 1)
                want = scatter(sc, r, 1, sp, d, thr, ior, last_pdf, rng, no, nd, want_shadow,
                                    s_o, s_d, s_c);
            t.w.path[2 * p + 0] = make_float4(thr.x, thr.y, thr.z, ior);
            t.w.path[2 * p + 1] = make_float4(rad.x, rad.y, rad.z, last_pdf);
            rng_state = rng.state;
        }
        const uint32_t tag = (ci << kPathBits) | p;
        const uint32_t q = warp_append(t.w.counters + 0, want);
        if (want) {
            t.w.q_od[0][2 * q + 0] = make_float4(no.x, no.y, no.z, __uint_as_float(rng_state));
            t.w.q_od[0][2 * q + 1] = make_float4(nd.x, nd.y, nd.z, __uint_as_float(tag));
        }
        {
            const uint32_t sq = warp_append(t.w.counters + 2, want_shadow);
            if (want_shadow) {
                t.w.s_od[2 * sq + 0] = s_o;
                t.w.s_od[2 * sq + 1] = s_d;
                t.w.s_contrib[sq] = s_c;
                t.w.s_path[sq] = tag;
            }
        }
    }
}

// Closest hit for every entry of ray queue `qi` (persistent warps, counter w.counters[4]).
template <bool COUNT, bool TWO_LEVEL, bool ALPHA>
__global__ void __launch_bounds__(128, kTraceBlocksPerSM)
    k_trace(TickArgs t, int qi, unsigned long long* work_ctr, int sort) {
    const uint32_t n = t.w.counters[qi];
    TraceCounters ctr{0, 0, 0, 0, 0, 0};
    // with material-sorted shading: each hit's sort key, counted per block in shared memory
    __shared__ uint32_t key_count[kSortKeys];
    if (threadIdx.x < kSortKeys) key_count[threadIdx.x] = 0u;
    __syncthreads();
    const float4* q = t.w.q_od[qi];
    // the entry's chunk, from the tag in the direction's w
    auto chunk_of = [&](uint32_t i) -> const ChunkGPU& {
        return t.chunks[__float_as_uint(__ldg((const float*)&q[2 * i + 1] + 3)) >> kPathBits];
    };
    auto load = [&](uint32_t i, TraceState& s) {
        const float4 a = q[2 * i + 0];
        const float4 b = q[2 * i + 1];
        const ChunkGPU& c = t.chunks[__float_as_uint(b.w) >> kPathBits];
        s.nodes = c.nodes;
        s.tris_base = c.tris;
        s.tri_stride = c.tri_stride;
        s.insts = c.insts;
        s.mask = c.mask;
        trace_init(s, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), 0.0f, kRayTmax);
    };
    auto store = [&](uint32_t i, const Hit& h) {
        t.w.hit[2 * i + 0] =
            make_uint4(__float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v), h.prim);
        t.w.hit[2 * i + 1] = make_uint4(h.geom, h.inst, 0u, 0u);
        if (sort) {
            uint32_t key = 0u; // misses shade the environment
            if (h.geom != kNoInst) key = __ldg(&chunk_of(i).geom_key[h.geom]);
            t.w.keys[i] = (uint8_t)key;
            atomicAdd(&key_count[key], 1u);
        }
    };
    auto alpha = [&](uint32_t i, uint32_t g, uint32_t p, float u, float v) {
        return ALPHA && alpha_discard(t.scenes[chunk_of(i).scene], g, p, u, v);
    };
    trace_persistent<false, COUNT, TWO_LEVEL>(n, t.w.counters + 4, load, store, alpha, &ctr,
                                              t.w.counters + 3, t.refill_lanes,
                                              t.postpone_lanes);
    if (sort) {
        __syncthreads();
        if (threadIdx.x < kSortKeys && key_count[threadIdx.x])
            atomicAdd(t.w.counters + 8 + threadIdx.x, key_count[threadIdx.x]);
    }
    if (COUNT) {
        atomicAdd(work_ctr + 0, (unsigned long long)ctr.nodes);
        atomicAdd(work_ctr + 1, (unsigned long long)ctr.tris);
        if (ctr.node_steps) {
            atomicAdd(work_ctr + 4, (unsigned long long)ctr.node_steps);
            atomicAdd(work_ctr + 5, (unsigned long long)ctr.node_lanes);
        }
        if (ctr.tri_steps) {
            atomicAdd(work_ctr + 6, (unsigned long long)ctr.tri_steps);
            atomicAdd(work_ctr + 7, (unsigned long long)ctr.tri_lanes);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(t.w.stats + 0, (unsigned long long)n);
        atomicAdd(t.w.stats + 2, (unsigned long long)n);
    }
}

// Emission at the k-th path vertex, then scatter (k < L) into ray queue `qo`.
__global__ void __launch_bounds__(128, kShadeBlocksPerSM)
    k_shade(TickArgs t, int k, int qi, int qo, const uint32_t* __restrict__ perm) {
    const uint32_t n = t.w.counters[qi];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_round = (n + 31u) & ~31u;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_round; j += stride) {
        bool want = false, want_shadow = false;
        float3 no, nd;
        float4 s_o, s_d, s_c;
        uint32_t tag = 0, rng_state = 0;
        if (j < n) {
            const uint32_t i = perm ? __ldg(&perm[j]) : j;
            // the entry's sector: the path's RNG state and the tag ride in the w components; a
            // surface point comes from the hit's vertices, and an environment point's position
            // is never read here (it does not scatter)
            const float4 qa = t.w.q_od[qi][2 * i + 0];
            const float4 qb = t.w.q_od[qi][2 * i + 1];
            tag = __float_as_uint(qb.w);
            const uint32_t p = tag & kPathMask;
            const ChunkGPU& c = t.chunks[tag >> kPathBits];
            const ReqGPU& r = t.reqs[c.req];
            const DevScene& sc = t.scenes[c.scene];
            const float3 o = f3(0.f, 0.f, 0.f), d = f3(qb.x, qb.y, qb.z);
            const uint4 h0 = t.w.hit[2 * i + 0], h1 = t.w.hit[2 * i + 1];
            const float4 h = make_float4(__uint_as_float(h0.x), __uint_as_float(h0.y),
                                         __uint_as_float(h0.z), __uint_as_float(h0.w));
            const uint32_t geom = h1.x;
            const float4 t4 = t.w.path[2 * p + 0], r4 = t.w.path[2 * p + 1];
            float3 thr = f3(t4.x, t4.y, t4.z), rad = f3(r4.x, r4.y, r4.z);
            float ior = t4.w, last_pdf = r4.w;
            Pcg rng{__float_as_uint(qa.w)};
            SPd sp;
            // a miss: the map coordinates serve the radiance and, with NEE, the MIS density
            const bool miss = geom == 0xFFFFFFFFu || geom >= sc.geom_count;
            float eu = 0.f, ev = 0.f;
            if (miss) {
                if (sc.ew) env_uv(sc, d, eu, ev);
                sp = env_sp_uv(sc, o, d, eu, ev);
            } else {
                sp = surface_sp(sc, o, d, geom, h0.w, h.y, h.z, h1.y);
            }
            const bool scatters = k < (int)r.max_len;
            sp.has_material = sp.has_material && scatters;
            float3 e = thr * sp.emission;
            if ((r.flags & kReqNee) && !all_zero(e)) {
                float pl = 0.f;
                if (sp.env) pl = sc.p_env * (miss ? env_pdf_uv(sc, eu, ev) : env_pdf(sc, d));
                else if (sp.emissive) pl = tri_light_pdf(sc, sp.emission, h.x * h.x, dot(d, sp.fn));
                e = e * power_heuristic(last_pdf, pl);
            }
            rad = rad + e;
            if (scatters)
                want = scatter(sc, r, k, sp, d, thr, ior, last_pdf, rng, no, nd, want_shadow,
                                    s_o, s_d, s_c);
            t.w.path[2 * p + 0] = make_float4(thr.x, thr.y, thr.z, ior);
            t.w.path[2 * p + 1] = make_float4(rad.x, rad.y, rad.z, last_pdf);
            rng_state = rng.state;
        }
        const uint32_t q = warp_append(t.w.counters + qo, want);
        if (want) {
            t.w.q_od[qo][2 * q + 0] = make_float4(no.x, no.y, no.z, __uint_as_float(rng_state));
            t.w.q_od[qo][2 * q + 1] = make_float4(nd.x, nd.y, nd.z, __uint_as_float(tag));
        }
        {
            const uint32_t sq = warp_append(t.w.counters + 2, want_shadow);
            if (want_shadow) {
                t.w.s_od[2 * sq + 0] = s_o;
                t.w.s_od[2 * sq + 1] = s_d;
                t.w.s_contrib[sq] = s_c;
                t.w.s_path[sq] = tag;
            }
        }
    }
}

// The entries in key order (a stable-within-tile counting sort): the traversal wrote each
// entry's key and the per-key totals; each block takes tiles of kSortTile consecutive entries,
// ranks them per key with warp ballots, reserves its ranges with one atomic per key and tile, and
// writes the permutation. The order of the tiles within a key is not deterministic (shading does
// not depend on it).
constexpr uint32_t kSortTile = 2048; // 256 threads x 8 entries
__global__ void __launch_bounds__(256) k_sort_scatter(TickArgs t, int qi, uint32_t* perm) {
    const uint32_t n = qi < 0 ? t.hdr->n_paths : t.w.counters[qi]; // qi < 0: the tick's paths
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __shared__ uint32_t warp_count[8][kSortKeys]; // then each warp's offset within the tile
    __shared__ uint32_t tile_base[kSortKeys];
    uint32_t key_base[kSortKeys];
    uint32_t acc = 0;
#pragma unroll
    for (int k = 0; k < kSortKeys; ++k) {
        key_base[k] = acc;
        acc += t.w.counters[8 + k];
    }
    for (uint32_t tile = blockIdx.x; tile * kSortTile < n; tile += gridDim.x) {
        // this warp's 256 consecutive entries: 8 rounds of 32
        const uint32_t first = tile * kSortTile + warp * 256u;
        uint8_t key[8];
        uint32_t count[kSortKeys] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const uint32_t i = first + 32u * r + lane;
            key[r] = i < n ? t.w.keys[i] : (uint8_t)0xFF;
#pragma unroll
            for (int k = 0; k < kSortKeys; ++k)
                count[k] += __popc(__ballot_sync(0xFFFFFFFFu, key[r] == k));
        }
        if (lane < kSortKeys) {
            uint32_t c = 0;
#pragma unroll
            for (int k = 0; k < kSortKeys; ++k)
                if (k == (int)lane) c = count[k];
            warp_count[warp][lane] = c;
        }
        __syncthreads();
        if (threadIdx.x < kSortKeys) {
            const uint32_t k = threadIdx.x;
            uint32_t run = 0;
            for (int w = 0; w < 8; ++w) {
                const uint32_t c = warp_count[w][k];
                warp_count[w][k] = run;
                run += c;
            }
            tile_base[k] = run ? key_base[k] + atomicAdd(t.w.counters + 12 + k, run) : 0u;
        }
        __syncthreads();
        uint32_t at[kSortKeys];
#pragma unroll
        for (int k = 0; k < kSortKeys; ++k) at[k] = tile_base[k] + warp_count[warp][k];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const uint32_t i = first + 32u * r + lane;
#pragma unroll
            for (int k = 0; k < kSortKeys; ++k) {
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, key[r] == k);
                if (key[r] == k) perm[at[k] + __popc(m & ((1u << lane) - 1u))] = i;
                at[k] += __popc(m);
            }
        }
        __syncthreads(); // warp_count and tile_base are reused by the next tile
    }
}

// Occlusion of the NEE queue; unoccluded contributions are added to their path (one shadow ray
// per path per bounce, so no two lanes write the same path).
template <bool TWO_LEVEL, bool ALPHA>
__global__ void __launch_bounds__(128, kTraceBlocksPerSM) k_shadow(TickArgs t) {
    const uint32_t n = t.w.counters[2];
    auto load = [&](uint32_t i, TraceState& s) {
        const ChunkGPU& c = t.chunks[__ldg(&t.w.s_path[i]) >> kPathBits];
        const float4 a = t.w.s_od[2 * i + 0];
        const float4 b = t.w.s_od[2 * i + 1];
        s.nodes = c.nodes;
        s.tris_base = c.tris;
        s.tri_stride = c.tri_stride;
        s.insts = c.insts;
        s.mask = c.mask;
        trace_init(s, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), 0.0f, a.w);
    };
    auto store = [&](uint32_t i, const Hit& h) {
        if (h.geom == 0xFFFFFFFFu) {
            const uint32_t p = t.w.s_path[i] & kPathMask;
            const float4 c = t.w.s_contrib[i];
            float4 r = t.w.path[2 * p + 1];
            r.x += c.x;
            r.y += c.y;
            r.z += c.z;
            t.w.path[2 * p + 1] = r;
        }
    };
    auto alpha = [&](uint32_t i, uint32_t g, uint32_t p, float u, float v) {
        return ALPHA && alpha_discard(t.scenes[t.chunks[__ldg(&t.w.s_path[i]) >> kPathBits].scene],
                                      g, p, u, v);
    };
    trace_persistent<true, false, TWO_LEVEL>(n, t.w.counters + 5, load, store, alpha, nullptr,
                                             t.w.counters + 3, t.refill_lanes, t.postpone_lanes);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(t.w.stats + 0, (unsigned long long)n);
        atomicAdd(t.w.stats + 1, (unsigned long long)n);
    }
}

// Per-pixel mean and mean squared luminance over the samples (render_pt.slang:110-129); one warp
// per pixel, lanes stride the samples, fixed shuffle tree: a deterministic summation order.
__global__ void __launch_bounds__(128) k_finalize(TickArgs t) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t n = t.hdr->n_pix, nc = t.hdr->n_chunks;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += warps) {
        const ChunkGPU c = t.chunks[chunk_by_slot(t.chunks, nc, q)];
        const ReqGPU& r = t.reqs[c.req];
        const uint32_t S = c.spp;
        const uint64_t base = (uint64_t)c.path_base + (uint64_t)(q - c.slot_base) * S;
        float cr = 0.f, cg = 0.f, cb = 0.f, m = 0.f;
        // per-sample demodulation (render_pt.slang:105-116): 1 unless "demodulate albedo"
        const float4* pc = t.w.pix + kPixFloat4 * q;
        const float ax = pc[3].w, ay = pc[4].w, az = pc[5].w;
        const bool demod = (r.flags & kReqDemodulate) != 0u;
        for (uint32_t s = lane; s < S; s += 32u) {
            float4 v = t.w.path[2 * (base + s) + 1];
            if (demod) {
                v.x = v.x / ax;
                v.y = v.y / ay;
                v.z = v.z / az;
            }
            if (isfinite(v.x) && isfinite(v.y) && isfinite(v.z)) {
                cr += v.x;
                cg += v.y;
                cb += v.z;
                const float l = yuv_luminance(f3(v.x, v.y, v.z));
                m += l * l;
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            cr += __shfl_xor_sync(0xFFFFFFFFu, cr, off);
            cg += __shfl_xor_sync(0xFFFFFFFFu, cg, off);
            cb += __shfl_xor_sync(0xFFFFFFFFu, cb, off);
            m += __shfl_xor_sync(0xFFFFFFFFu, m, off);
        }
        if (lane == 0) {
            const float inv = S > 0 ? 1.0f / (float)S : 0.f;
            r.out[c.pix_first + (q - c.slot_base)] =
                make_float4(cr * inv, cg * inv, cb * inv, m * inv);
        }
    }
}

std::atomic<uint64_t> g_generation{0};
void new_generation(Work& w) { w.generation = ++g_generation; }

// On failure p is null (never a stale address).
template <class T> cudaError_t alloc(T*& p, uint64_t n, uint64_t& bytes) {
    bytes += n * sizeof(T);
    void* q = nullptr;
    const cudaError_t e = device_malloc(&q, n * sizeof(T) + 16);
    p = e == cudaSuccess ? (T*)q : nullptr;
    return e;
}
template <class T> void release(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

ReqGPU to_req(const BatchItem& it, uint32_t scene_index) {
    const gbpt_camera& c = it.camera;
    const gbpt_render_params& p = it.params;
    ReqGPU r{};
    r.cam.pos = make_float3(c.position[0], c.position[1], c.position[2]);
    r.cam.U = make_float3(c.U[0], c.U[1], c.U[2]);
    r.cam.V = make_float3(c.V[0], c.V[1], c.V[2]);
    r.cam.W = make_float3(c.W[0], c.W[1], c.W[2]);
    r.cam.near_plane = c.near_plane;
    r.cam.far_plane = c.far_plane;
    r.cam.jx = c.jitter[0];
    r.cam.jy = c.jitter[1];
    r.width = p.width;
    r.height = p.height;
    r.spp = (uint32_t)p.spp;
    r.max_len = (uint32_t)p.max_path_length;
    const bool nee = p.nee && (it.scene->n_lights > 0 || it.scene->env != nullptr);
    r.flags = (p.emission_on_primary ? kReqEmission : 0u) | (nee ? kReqNee : 0u) |
              (p.demodulate_albedo ? kReqDemodulate : 0u);
    r.mask = p.instance_mask & 0xFFu;
    r.frame = p.frame;
    r.rr_depth = p.rr_depth;
    r.scene = scene_index;
    r.pixels = it.pixels_device;
    r.out = it.out_device;
    return r;
}

} // namespace

int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 152;
    }
    return n;
}

void work_free(Work& w) {
    if (w.fixed) {
        w = Work{};
        return;
    }
    void* ptrs[] = {w.path,    w.q_od[0],   w.q_od[1], w.hit,     w.s_od,  w.s_contrib, w.s_path,
                    w.pix,     w.pix_id,    w.out,    w.counters, w.stats,    w.tables,
                    w.keys,    w.perm};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    w = Work{};
}

int work_reserve(Work& w, uint64_t paths, uint64_t pixels) {
    if (w.fixed) return (paths <= w.path_cap && pixels <= w.pixel_cap) ? GBPT_OK : GBPT_ERR_NO_MEMORY;
    if (!w.counters || !w.stats) {
        uint64_t b = 0;
        release(w.counters);
        release(w.stats);
        if (alloc(w.counters, 16, b) != cudaSuccess || alloc(w.stats, 8, b) != cudaSuccess) {
            release(w.counters);
            release(w.stats);
            return GBPT_ERR_NO_MEMORY;
        }
        new_generation(w);
        cudaMemset(w.counters, 0, 16 * sizeof(uint32_t));
        cudaMemset(w.stats, 0, 8 * sizeof(unsigned long long));
        w.bytes += b;
    }
    if (paths > w.path_cap) {
        auto release_paths = [&w]() {
            release(w.path);
            release(w.q_od[0]);
            release(w.q_od[1]);
            release(w.hit);
            release(w.s_od);
            release(w.s_contrib);
            release(w.s_path);
            release(w.keys);
            release(w.perm);
            w.path_cap = 0;
        };
        release_paths();
        new_generation(w);
        uint64_t b = 0;
        bool ok = alloc(w.path, 2 * paths, b) == cudaSuccess &&
                  alloc(w.q_od[0], 2 * paths, b) == cudaSuccess &&
                  alloc(w.q_od[1], 2 * paths, b) == cudaSuccess &&
                  alloc(w.hit, 2 * paths, b) == cudaSuccess &&
                  alloc(w.s_od, 2 * paths, b) == cudaSuccess &&
                  alloc(w.s_contrib, paths, b) == cudaSuccess &&
                  alloc(w.s_path, paths, b) == cudaSuccess &&
                  alloc(w.keys, paths, b) == cudaSuccess && alloc(w.perm, paths, b) == cudaSuccess;
        if (!ok) {
            release_paths();
            return GBPT_ERR_NO_MEMORY;
        }
        w.path_cap = paths;
        w.bytes += b;
    }
    if (pixels > w.pixel_cap) {
        release(w.pix);
        w.pixel_cap = 0;
        new_generation(w);
        uint64_t b = 0;
        if (alloc(w.pix, kPixFloat4 * pixels, b) != cudaSuccess) return GBPT_ERR_NO_MEMORY;
        w.pixel_cap = pixels;
        w.bytes += b;
    }
    return GBPT_OK;
}

namespace {

// The tick tables in w.tables, for a tick of at most `cap` chunks: header, then the tick's
// requests, scenes and chunks (each a tick-local table), at fixed offsets so that a captured
// graph reads every tick from the same addresses.
struct SlotLayout {
    uint32_t cap;
    uint64_t reqs, scenes, chunks, end;
};
SlotLayout slot_layout(uint32_t cap) {
    auto up = [](uint64_t x) { return (x + 255) & ~uint64_t(255); };
    SlotLayout l;
    l.cap = cap;
    l.reqs = 256;
    l.scenes = l.reqs + up((uint64_t)cap * sizeof(ReqGPU));
    l.chunks = l.scenes + up((uint64_t)cap * sizeof(DevScene));
    l.end = l.chunks + (uint64_t)cap * sizeof(ChunkGPU);
    return l;
}
// the most chunks per tick that `bytes` of tables hold
uint32_t slot_capacity(uint64_t bytes) {
    uint32_t cap = kMaxChunks;
    while (cap > 0 && slot_layout(cap).end > bytes) --cap;
    return cap;
}

int tables_reserve(Work& w, uint64_t need) {
    if (need <= w.tables_bytes) return GBPT_OK;
    if (w.fixed) return GBPT_ERR_NO_MEMORY;
    if (w.tables) cudaFree(w.tables);
    w.tables = nullptr;
    w.tables_bytes = 0;
    const uint64_t cap = std::max<uint64_t>(need + need / 2, 64 << 10);
    new_generation(w);
    if (device_malloc(&w.tables, cap) != cudaSuccess) {
        w.tables = nullptr;
        return GBPT_ERR_NO_MEMORY;
    }
    w.tables_bytes = cap;
    w.bytes += cap;
    return GBPT_OK;
}

struct TickPlan {
    uint32_t chunk_first, n_chunks, n_pix, n_paths, max_len;
    bool nee;
    bool sort; // material-sorted shading (some request asked for it and the Work has the buffers)
    bool two_level; // some chunk's scene is instanced: the two-level traversal variants
    bool alpha;     // some chunk's scene has alpha-tested geometry: the alpha-test variants
};

// Grid-stride kernels get exactly the blocks that are resident at once: every block strides over
// the same share of the work, so a second partial wave of blocks would only add a tail.
struct Grids {
    int grid;    // grid-stride kernels without a register budget (finalize, material sort)
    int trace;   // persistent traversal: the blocks resident at once
    int trace_c;
    int shadow;
    int primary; // k_primary, k_shade_primary, k_shade: their resident blocks
    int shade_p;
    int shade;
};
Grids launch_grids() {
    Grids g;
    g.grid = num_sms() * 8;
    // the two-level and alpha variants have the same launch bounds, hence the same residency
    g.trace = persistent_grid(k_trace<false, false, false>);
    g.trace_c = persistent_grid(k_trace<true, false, false>);
    g.shadow = persistent_grid(k_shadow<false, false>);
    g.primary = persistent_grid(k_primary);
    g.shade_p = persistent_grid(k_shade_primary);
    g.shade = persistent_grid(k_shade);
    return g;
}

// The traversal variants of a tick: work counters, two-level scenes, alpha-tested geometry (the
// variants without a feature leave its code out; they find the same hits on scenes without it).
void launch_trace(const TickArgs& ta, const TickPlan& tp, const Grids& g, int qi,
                  unsigned long long* work_ctr, cudaStream_t st) {
    const int gr = work_ctr ? g.trace_c : g.trace;
    const int so = tp.sort ? 1 : 0;
    switch ((work_ctr ? 4 : 0) | (tp.two_level ? 2 : 0) | (tp.alpha ? 1 : 0)) {
    case 0: k_trace<false, false, false><<<gr, 128, 0, st>>>(ta, qi, nullptr, so); break;
    case 1: k_trace<false, false, true><<<gr, 128, 0, st>>>(ta, qi, nullptr, so); break;
    case 2: k_trace<false, true, false><<<gr, 128, 0, st>>>(ta, qi, nullptr, so); break;
    case 3: k_trace<false, true, true><<<gr, 128, 0, st>>>(ta, qi, nullptr, so); break;
    case 4: k_trace<true, false, false><<<gr, 128, 0, st>>>(ta, qi, work_ctr, so); break;
    case 5: k_trace<true, false, true><<<gr, 128, 0, st>>>(ta, qi, work_ctr, so); break;
    case 6: k_trace<true, true, false><<<gr, 128, 0, st>>>(ta, qi, work_ctr, so); break;
    default: k_trace<true, true, true><<<gr, 128, 0, st>>>(ta, qi, work_ctr, so); break;
    }
}

void launch_shadow(const TickArgs& ta, const TickPlan& tp, const Grids& g, cudaStream_t st) {
    switch ((tp.two_level ? 2 : 0) | (tp.alpha ? 1 : 0)) {
    case 0: k_shadow<false, false><<<g.shadow, 128, 0, st>>>(ta); break;
    case 1: k_shadow<false, true><<<g.shadow, 128, 0, st>>>(ta); break;
    case 2: k_shadow<true, false><<<g.shadow, 128, 0, st>>>(ta); break;
    default: k_shadow<true, true><<<g.shadow, 128, 0, st>>>(ta); break;
    }
}

// The kernel sequence of one tick; returns the number of kernel launches. Counter words
// ([0], [1] ray queues, [2] shadow queue, [4], [5] fetch cursors) are cleared on the stream
// before their producer runs; the error flag ([3]) is left for the caller to read.
// With fixed_grid every launch gets the full grid whatever the tick's size (a graph replays any
// tick of the same shape); the kernels stride over the sizes in the tick header.
uint64_t enqueue_tick(const TickArgs& ta, const TickPlan& tp, const Grids& g, cudaStream_t st,
                      Profile* prof, unsigned long long* work_ctr, bool fixed_grid) {
    uint32_t* ctr = ta.w.counters;
    const bool nee = tp.nee;
    const uint32_t L = tp.max_len;
    const uint64_t pix = fixed_grid ? ~0ull >> 8 : tp.n_pix;
    const uint64_t paths = fixed_grid ? ~0ull >> 8 : tp.n_paths;
    uint64_t nl = 0;
    cudaMemsetAsync(ctr, 0, 3 * sizeof(uint32_t), st);
    const int pgrid = (int)std::min<uint64_t>((pix + 127) / 128, (uint64_t)g.primary);
    if (tp.sort) cudaMemsetAsync(ctr + 8, 0, 8 * sizeof(uint32_t), st); // key counts, cursors
    int ev = prof->begin(st, 3);
    k_primary<<<pgrid, 128, 0, st>>>(ta, tp.sort ? 1 : 0);
    prof->end(st, ev);
    const uint32_t* pperm = nullptr;
    if (tp.sort) {
        ev = prof->begin(st, 1);
        k_sort_scatter<<<g.grid / 2, 256, 0, st>>>(ta, -1, ta.w.perm);
        prof->end(st, ev);
        pperm = ta.w.perm;
        nl += 1;
    }
    const int sgrid = (int)std::min<uint64_t>((paths + 127) / 128, (uint64_t)g.shade_p);
    ev = prof->begin(st, 1);
    k_shade_primary<<<sgrid, 128, 0, st>>>(ta, pperm);
    prof->end(st, ev);
    nl += 2;
    if (nee) {
        cudaMemsetAsync(ctr + 5, 0, sizeof(uint32_t), st);
        ev = prof->begin(st, 2);
        launch_shadow(ta, tp, g, st);
        prof->end(st, ev);
        cudaMemsetAsync(ctr + 2, 0, sizeof(uint32_t), st);
        nl += 1;
    }
    int qi = 0;
    for (uint32_t k = 2; k <= L; ++k) {
        const int qo = qi ^ 1;
        cudaMemsetAsync(ctr + 4, 0, sizeof(uint32_t), st);
        if (tp.sort) cudaMemsetAsync(ctr + 8, 0, 8 * sizeof(uint32_t), st); // key counts, cursors
        ev = prof->begin(st, 0);
        launch_trace(ta, tp, g, qi, work_ctr, st);
        prof->end(st, ev);
        const uint32_t* perm = nullptr;
        if (tp.sort) {
            ev = prof->begin(st, 1);
            k_sort_scatter<<<g.grid / 2, 256, 0, st>>>(ta, qi, ta.w.perm);
            prof->end(st, ev);
            perm = ta.w.perm;
            nl += 1;
        }
        cudaMemsetAsync(ctr + qo, 0, sizeof(uint32_t), st);
        ev = prof->begin(st, 1);
        k_shade<<<g.shade, 128, 0, st>>>(ta, (int)k, qi, qo, perm);
        prof->end(st, ev);
        nl += 2;
        if (nee && k < L) {
            cudaMemsetAsync(ctr + 5, 0, sizeof(uint32_t), st);
            ev = prof->begin(st, 2);
            launch_shadow(ta, tp, g, st);
            prof->end(st, ev);
            cudaMemsetAsync(ctr + 2, 0, sizeof(uint32_t), st);
            nl += 1;
        }
        qi = qo;
    }
    ev = prof->begin(st, 3);
    k_finalize<<<(int)std::min<uint64_t>((pix * 32 + 127) / 128, (uint64_t)g.grid), 128, 0, st>>>(ta);
    prof->end(st, ev);
    return nl + 1;
}

} // namespace

uint64_t tick_table_bytes(uint32_t max_chunks) { return slot_layout(max_chunks).end; }

int Profile::begin(cudaStream_t st, int c) {
    if (level <= 0) return -1;
    if (2 * (used + 1) > ev.size()) {
        for (int k = 0; k < 2; ++k) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            ev.push_back(e);
        }
    }
    const int pair = (int)used++;
    cls.push_back(c);
    cudaEventRecord(ev[2 * pair], st);
    return pair;
}

void Profile::end(cudaStream_t st, int pair) {
    if (pair >= 0) cudaEventRecord(ev[2 * pair + 1], st);
}

void Profile::destroy() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    ev.clear();
    reset();
}

void TickEngine::release() {
    for (const Graph& g : graphs) cudaGraphExecDestroy(g.exec);
    graphs.clear();
    graph_generation = 0;
}

int tick_enqueue(TickEngine& e, TickItem* const* items, uint32_t n_items, uint64_t* n_paths,
                 std::vector<uint32_t>* done, uint64_t* launches, Profile* prof,
                 unsigned long long* work_ctr) {
    Profile dummy;
    if (!prof) prof = &dummy;
    *n_paths = 0;
    Work& w = *e.work;
    const cudaStream_t st = e.stream;
    int rc;
    // tick tables: the full slot, or as many chunks as a fixed Work's table area holds
    if (!w.fixed && (rc = tables_reserve(w, slot_layout(kMaxChunks).end)) != GBPT_OK) return rc;
    const uint32_t cap = slot_capacity(w.tables_bytes);
    if (cap == 0) return GBPT_ERR_NO_MEMORY;
    const SlotLayout lay = slot_layout(cap);
    const uint64_t wave = w.fixed ? std::min<uint64_t>(e.wave, w.path_cap) : e.wave;
    if (wave == 0 || wave > kMaxWavePaths) return GBPT_ERR_INVALID;

    // Plan: FIFO over the items, whole pixels until the wave is full, at most one chunk per
    // item; an item that does not fit stops the plan, so later items never overtake it.
    e.stage.assign(lay.end, 0);
    unsigned char* sb = e.stage.data();
    ReqGPU* reqs = (ReqGPU*)(sb + lay.reqs);
    DevScene* scenes = (DevScene*)(sb + lay.scenes);
    ChunkGPU* chunks = (ChunkGPU*)(sb + lay.chunks);
    e.scene_ptrs.clear();
    TickPlan tp{0, 0, 0, 0, 1, false, false, false, false};
    uint64_t paths = 0, pix = 0;
    for (uint32_t i = 0; i < n_items && tp.n_chunks < cap; ++i) {
        TickItem& it = *items[i];
        const uint32_t S = (uint32_t)std::max(it.params.spp, 0);
        if (S == 0 || it.cursor >= it.pixel_count) continue;
        if (S > wave) return GBPT_ERR_INVALID;
        const uint64_t fit = std::min<uint64_t>(it.pixel_count - it.cursor, (wave - paths) / S);
        if (fit == 0) break;
        uint32_t si = 0;
        while (si < e.scene_ptrs.size() && e.scene_ptrs[si] != it.scene) ++si;
        if (si == e.scene_ptrs.size()) {
            e.scene_ptrs.push_back(it.scene);
            scenes[si] = make_dev_scene(*it.scene);
        }
        const uint32_t ri = tp.n_chunks;
        reqs[ri] = to_req(it, si);
        ChunkGPU& c = chunks[ri];
        c.req = ri;
        c.scene = si;
        c.pix_first = it.cursor;
        c.n_pix = (uint32_t)fit;
        c.slot_base = (uint32_t)pix;
        c.path_base = (uint32_t)paths;
        c.spp = S;
        c.mask = reqs[ri].mask;
        c.nodes = scenes[si].nodes;
        c.tris = scenes[si].tris;
        c.tri_stride = scenes[si].tri_stride;
        c.insts = scenes[si].n_inst ? scenes[si].inst : nullptr;
        c.geom_key = (const uint8_t*)it.scene->geom_key;
        tp.two_level |= scenes[si].n_inst != 0u;
        tp.alpha |= it.scene->alpha;
        ++tp.n_chunks;
        paths += fit * S;
        pix += fit;
        tp.max_len = std::max(tp.max_len, reqs[ri].max_len);
        tp.nee |= (reqs[ri].flags & kReqNee) != 0u;
        tp.sort |= it.params.sort_materials != 0;
        it.cursor += (uint32_t)fit;
        if (done && it.cursor == it.pixel_count) done->push_back(i);
    }
    if (tp.n_chunks == 0) return GBPT_OK;
    tp.n_pix = (uint32_t)pix;
    tp.n_paths = (uint32_t)paths;
    *(TickHeader*)sb = TickHeader{tp.n_chunks, tp.n_pix, tp.n_paths, 0u};

    // work buffers: a whole wave when graphs replay the tick (their pointers must not move)
    bool graph = e.use_graphs && prof->level == 0;
    if ((rc = work_reserve(w, graph ? wave : paths, graph ? wave : pix)) != GBPT_OK) return rc;
    tp.sort = tp.sort && w.perm != nullptr;
    unsigned char* tb = (unsigned char*)w.tables;
    if (cudaMemcpyAsync(tb, sb, lay.chunks + tp.n_chunks * sizeof(ChunkGPU), cudaMemcpyHostToDevice,
                        st) != cudaSuccess)
        return GBPT_ERR_CUDA;
    TickArgs ta;
    ta.hdr = (const TickHeader*)tb;
    ta.reqs = (const ReqGPU*)(tb + lay.reqs);
    ta.scenes = (const DevScene*)(tb + lay.scenes);
    ta.chunks = (const ChunkGPU*)(tb + lay.chunks);
    ta.w = w;
    ta.refill_lanes = (int)e.sched.refill_lanes;
    ta.postpone_lanes = (int)e.sched.postpone_lanes;
    if (e.grids[0] == 0) {
        const Grids g = launch_grids();
        static_assert(sizeof(Grids) == sizeof(e.grids), "grid cache");
        std::memcpy(e.grids, &g, sizeof(g));
    }
    Grids grids;
    std::memcpy(&grids, e.grids, sizeof(grids));
    if (e.sched.blocks_per_sm > 0) {
        const int cap = (int)e.sched.blocks_per_sm * num_sms();
        grids.trace = std::min(grids.trace, cap);
        grids.trace_c = std::min(grids.trace_c, cap);
        grids.shadow = std::min(grids.shadow, cap);
    }
    uint64_t nl = 0;
    if (graph) {
        if (e.graph_generation != w.generation) {
            e.release();
            e.graph_generation = w.generation;
        }
        const uint32_t shape =
            tp.max_len * 16u + (tp.nee ? 1u : 0u) + (tp.sort ? 2u : 0u) + (tp.two_level ? 4u : 0u) +
            (tp.alpha ? 8u : 0u);
        const TickEngine::Graph* found = nullptr;
        for (const auto& g : e.graphs)
            if (g.shape == shape) found = &g;
        if (!found) {
            // one graph per tick shape: the kernel sequence depends on the path length and the
            // estimator only; sizes and requests come from the tables at fixed addresses
            cudaGraph_t g = nullptr;
            cudaGraphExec_t exec = nullptr;
            if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return GBPT_ERR_CUDA;
            const uint64_t n_launch = enqueue_tick(ta, tp, grids, st, &dummy, nullptr, true);
            if (cudaStreamEndCapture(st, &g) != cudaSuccess || !g) return GBPT_ERR_CUDA;
            const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) return GBPT_ERR_CUDA;
            e.graphs.push_back(TickEngine::Graph{shape, exec, n_launch});
            found = &e.graphs.back();
        }
        if (cudaGraphLaunch(found->exec, st) != cudaSuccess) return GBPT_ERR_CUDA;
        nl = found->launches;
    } else {
        nl = enqueue_tick(ta, tp, grids, st, prof, prof->level >= 2 ? work_ctr : nullptr, false);
    }
    *n_paths = paths;
    if (launches) *launches += nl;
    return cudaGetLastError() == cudaSuccess ? GBPT_OK : GBPT_ERR_CUDA;
}

int render_batch(TickEngine& e, const BatchItem* items, uint32_t n_items, uint64_t* launches,
                 Profile* prof, unsigned long long* work_ctr, TickEngine* e2, cudaEvent_t fork,
                 cudaEvent_t join) {
    std::vector<TickItem> ti(n_items);
    std::vector<TickItem*> ptr(n_items);
    uint64_t max_spp = 0;
    for (uint32_t i = 0; i < n_items; ++i) {
        static_cast<BatchItem&>(ti[i]) = items[i];
        ptr[i] = &ti[i];
        max_spp = std::max<uint64_t>(max_spp, (uint64_t)std::max(items[i].params.spp, 0));
    }
    if (!e.work->fixed) e.wave = std::max<uint64_t>(e.wave, max_spp);
    if (!e2) {
        while (true) {
            uint64_t n = 0;
            const int rc =
                tick_enqueue(e, ptr.data(), n_items, &n, nullptr, launches, prof, work_ctr);
            if (rc != GBPT_OK) return rc;
            if (n == 0) return GBPT_OK;
        }
    }
    // two streams: ticks cover disjoint pixels, each over its own work buffers, so they only
    // share the scenes (read), the outputs (disjoint texels) and atomic counters
    e2->wave = e.wave;
    e2->sched = e.sched;
    if (cudaEventRecord(fork, e.stream) != cudaSuccess ||
        cudaStreamWaitEvent(e2->stream, fork, 0) != cudaSuccess)
        return GBPT_ERR_CUDA;
    int rc = GBPT_OK;
    for (uint64_t k = 0;; ++k) {
        uint64_t n = 0;
        rc = tick_enqueue((k & 1) ? *e2 : e, ptr.data(), n_items, &n, nullptr, launches, prof,
                          work_ctr);
        if (rc != GBPT_OK || n == 0) break;
    }
    const bool joined = cudaEventRecord(join, e2->stream) == cudaSuccess &&
                        cudaStreamWaitEvent(e.stream, join, 0) == cudaSuccess;
    return rc != GBPT_OK ? rc : (joined ? GBPT_OK : GBPT_ERR_CUDA);
}

int render_frame(const SceneGPU& scene, Work& w, const RenderArgs& args, cudaStream_t st,
                 uint64_t* launches, Profile* prof, unsigned long long* work_ctr, uint64_t wave,
                 Work* w2, cudaStream_t st2, cudaEvent_t fork, cudaEvent_t join,
                 const TraceSched& sched) {
    BatchItem it;
    it.scene = &scene;
    it.camera = args.camera;
    it.params = args.params;
    it.pixels_device = args.pixels_device;
    it.pixel_count = args.pixel_count;
    it.out_device = args.out_device;
    TickEngine e;
    e.work = &w;
    e.stream = st;
    e.sched = sched;
    if (wave) e.wave = wave;
    TickEngine e2;
    e2.work = w2;
    e2.stream = st2;
    e2.sched = sched;
    const int rc = render_batch(e, &it, 1, launches, prof, work_ctr, w2 ? &e2 : nullptr, fork,
                                join);
    e.release();
    e2.release();
    return rc;
}

// The primary shading points of the listed pixels (the first tick's k_primary only).
int primary_points(const SceneGPU& scene, Work& w, const RenderArgs& args, cudaStream_t st,
                   float* out_device) {
    const uint32_t P = args.pixel_count;
    int rc = work_reserve(w, std::max<uint64_t>(P, 1), std::max<uint64_t>(P, 1));
    if (rc != GBPT_OK) return rc;
    const SlotLayout lay = slot_layout(1);
    if ((rc = tables_reserve(w, lay.end)) != GBPT_OK) return rc;
    BatchItem it;
    it.scene = &scene;
    it.camera = args.camera;
    it.params = args.params;
    it.pixels_device = args.pixels_device;
    it.pixel_count = P;
    it.out_device = nullptr;
    unsigned char* tb = (unsigned char*)w.tables;
    TickHeader* d_hdr = (TickHeader*)tb;
    ReqGPU* d_reqs = (ReqGPU*)(tb + lay.reqs);
    DevScene* d_scenes = (DevScene*)(tb + lay.scenes);
    ChunkGPU* d_chunks = (ChunkGPU*)(tb + lay.chunks);
    const ReqGPU r = to_req(it, 0);
    const DevScene s = make_dev_scene(scene);
    ChunkGPU c{};
    c.req = 0;
    c.scene = 0;
    c.n_pix = P;
    c.spp = 1;
    c.mask = r.mask;
    c.nodes = s.nodes;
    c.tris = s.tris;
    c.tri_stride = s.tri_stride;
    const TickHeader hdr{1u, P, P, 0u};
    cudaMemcpyAsync(d_reqs, &r, sizeof(r), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_scenes, &s, sizeof(s), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_chunks, &c, sizeof(c), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_hdr, &hdr, sizeof(hdr), cudaMemcpyHostToDevice, st);
    TickArgs ta;
    ta.scenes = d_scenes;
    ta.reqs = d_reqs;
    ta.chunks = d_chunks;
    ta.hdr = d_hdr;
    ta.w = w;
    k_primary<<<(P + 127) / 128, 128, 0, st>>>(ta, 0);
    // the first 6 float4 of every cached point: the gbpt_debug_primary_points layout
    if (cudaMemcpy2DAsync(out_device, 6 * sizeof(float4), w.pix, kPixFloat4 * sizeof(float4),
                          6 * sizeof(float4), P, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return GBPT_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? GBPT_OK : GBPT_ERR_CUDA;
}

} // namespace gbpt

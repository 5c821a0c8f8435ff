// Wavefront kernels of the `pt` path and the host loop that drives them for one frame.
//
// merian runs one ray-generation thread per pixel that loops over samples and bounces
// (render_pt.slang:92-130, trace_path :24-90) on RT cores. Here one frame is processed in waves of
// (pixel, sample) paths held in SoA buffers in HBM:
//   primary   : camera ray + closest hit + primary shading point, once per pixel (the GBuffer's hit,
//               barycentrics rounded to half as the GBuffer stores them, gbuffer.slang:40-60)
//   shade<1>  : per path: RNG seed pcg4d16(pixel, frame, sample), emission on primary, scatter
//   loop k = 2..L: trace (closest hit of the ray queue) -> shade<k> (emission, Russian roulette,
//               next-event estimation, BSDF sample, ray append) -> shadow (any hit of the NEE queue)
//   finalize  : per pixel, samples summed in a fixed order, NaN/Inf samples dropped but counted
// Queue appends are warp-aggregated (one atomic per warp). Nothing on the host waits between
// kernels, so a frame is a fixed launch sequence on one stream.
#include "device_scene.cuh"
#include "runtime.h"

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <type_traits>

namespace gbpt {

std::string cuda_error_string(cudaError_t e) { return std::string(cudaGetErrorString(e)); }

namespace {

int g_num_sms = 0;
int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 152;
    }
    return g_num_sms;
}

DevScene make_dev_scene(const SceneGPU& s) {
    DevScene d{};
    d.nodes = (const uint4*)s.nodes;
    d.tris = (const float4*)s.tris;
    d.verts = (const uint32_t*)s.verts;
    d.idx = (const uint32_t*)s.idx;
    d.geoms = (const GeomGPU*)s.geoms;
    d.mats = (const float4*)s.mats;
    d.geom_count = s.geom_count;
    d.env = (const float4*)s.env;
    d.ew = s.env ? s.ew : 0u;
    d.eh = s.env ? s.eh : 0u;
    for (int i = 0; i < 9; ++i) d.env_m[i] = s.env_m[i];
    d.env_intensity = s.env_intensity;
    d.env_marg = (const float*)s.env_marg;
    d.env_cond = (const float*)s.env_cond;
    d.env_func = (const float*)s.env_func;
    d.env_func_int = s.env_func_int;
    d.light_tris = (const float4*)s.light_tris;
    d.light_cdf = (const float*)s.light_cdf;
    d.n_lights = s.n_lights;
    d.light_total = s.light_total;
    d.p_env = d.ew ? (s.n_lights ? 0.5f : 1.0f) : 0.0f;
    return d;
}

GBPT_DI uint32_t warp_append(uint32_t* counter, bool want) {
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, want);
    if (m == 0u) return 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return want ? base + __popc(m & ((1u << lane) - 1u)) : 0xFFFFFFFFu;
}

// ---- shading points (scene.slang:312-498) -----------------------------------------------------------
struct SPd {
    float3 pos;
    uint32_t enc_fn;
    float3 fn;        // exact face normal (FlipFacing applied), for light pdfs
    float3 emission;
    Frame frame;
    uint32_t mat;
    bool has_material;
    bool front;
    bool emissive;
    bool env;
};

GBPT_DI SPd env_sp(const DevScene& sc, float3 o, float3 d) {
    SPd sp;
    sp.pos = o + d * kEnvDistance;
    sp.enc_fn = encode_normal(-d);
    sp.fn = -d;
    sp.emission = env_eval(sc, d);
    sp.frame = frame_from_normal(-d);
    sp.mat = 0;
    sp.has_material = false;
    sp.front = true;
    sp.emissive = false;
    sp.env = true;
    return sp;
}

GBPT_DI void load_vertex(const DevScene& sc, uint32_t vi, float3& p, uint32_t& en, uint32_t& uv,
                         uint32_t& et) {
    const uint2* v = (const uint2*)(sc.verts + 6ull * vi);
    const uint2 a = __ldg(v), b = __ldg(v + 1), c = __ldg(v + 2);
    p = f3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(b.x));
    en = b.y;
    uv = c.x;
    et = c.y;
}

GBPT_DI SPd surface_sp(const DevScene& sc, float3 o, float3 d, uint32_t geom, uint32_t prim,
                       float bu, float bv) {
    const GeomGPU g = sc.geoms[geom];
    if (g.flags & GBPT_MESH_USE_ENV_MAP) return env_sp(sc, o, d);
    const uint32_t tri = g.first_triangle + prim;
    const uint32_t i0 = g.first_vertex + __ldg(&sc.idx[3 * tri + 0]);
    const uint32_t i1 = g.first_vertex + __ldg(&sc.idx[3 * tri + 1]);
    const uint32_t i2 = g.first_vertex + __ldg(&sc.idx[3 * tri + 2]);
    float3 p0, p1, p2;
    uint32_t n0, n1, n2, uv0, uv1, uv2, t0, t1, t2;
    load_vertex(sc, i0, p0, n0, uv0, t0);
    load_vertex(sc, i1, p1, n1, uv1, t1);
    load_vertex(sc, i2, p2, n2, uv2, t2);
    const float b0 = 1.0f - bu - bv, b1 = bu, b2 = bv;
    const float3 pos = (b0 * p0 + b1 * p1) + b2 * p2;
    const float3 e01 = p1 - p0, e02 = p2 - p0;
    float3 fn = normalize(cross(e01, e02));
    if (g.flags & GBPT_MESH_FLIP_FACING) fn = -fn;
    float3 vn;
    if (g.flags & GBPT_MESH_FLAT_SHADING) {
        vn = fn;
    } else {
        vn = normalize((b0 * decode_normal(n0) + b1 * decode_normal(n1)) + b2 * decode_normal(n2));
    }
    Frame frame;
    if (g.flags & GBPT_MESH_HAS_TANGENTS) {
        const float w0 = (t0 & 1u) ? -1.f : 1.f, w1 = (t1 & 1u) ? -1.f : 1.f,
                    w2 = (t2 & 1u) ? -1.f : 1.f;
        const float3 t = (b0 * decode_normal(t0 & ~1u) + b1 * decode_normal(t1 & ~1u)) +
                         b2 * decode_normal(t2 & ~1u);
        const float tw = (b0 * w0 + b1 * w1) + b2 * w2;
        frame = frame_from_tangent(vn, normalize(t), signf(tw));
    } else {
        const float d1x = half_lo(uv1) - half_lo(uv0), d1y = half_hi(uv1) - half_hi(uv0);
        const float d2x = half_lo(uv2) - half_lo(uv0), d2y = half_hi(uv2) - half_hi(uv0);
        const float det = d1x * d2y - d2x * d1y;
        if (fabsf(det) > 1e-8f) {
            const float winding = (g.flags & GBPT_MESH_FLIP_FACING) ? 1.f : -1.f;
            const float3 tg = (d2y * e01 - d1y * e02) / det;
            frame = frame_from_tangent(vn, tg, signf(det) * winding);
        } else {
            frame = frame_from_normal(vn);
        }
    }
    bool front = true;
    if (g.flags & GBPT_MESH_TWO_SIDED) {
        front = dot(-d, fn) >= 0.0f;
        if (!front) frame.n = -frame.n;
    }
    SPd sp;
    sp.pos = pos;
    sp.enc_fn = encode_normal(fn);
    sp.fn = fn;
    sp.mat = g.material;
    sp.front = front;
    sp.env = false;
    const float4 m0 = __ldg(&sc.mats[5 * g.material + 0]);
    const uint32_t model = __float_as_uint(m0.x);
    const float4 m2 = __ldg(&sc.mats[5 * g.material + 2]);
    const bool emits = model != GBPT_MATERIAL_DIFFUSE && (m2.y != 0.f || m2.z != 0.f || m2.w != 0.f);
    sp.emissive = emits && front;
    sp.emission = sp.emissive ? f3(m2.y, m2.z, m2.w) : f3(0.f, 0.f, 0.f);
    sp.frame = model == GBPT_MATERIAL_DIFFUSE ? reorthonormalize(frame) : frame;
    sp.has_material = true;
    return sp;
}

// OpenPBRMaterial::get_sample / DiffuseMaterial::get_sample for this shading point
GBPT_DI Material load_material(const DevScene& sc, uint32_t mid, bool front, float ior) {
    return material_from_record(__ldg(&sc.mats[5 * mid + 0]), __ldg(&sc.mats[5 * mid + 1]),
                                __ldg(&sc.mats[5 * mid + 2]), __ldg(&sc.mats[5 * mid + 3]), front,
                                ior);
}

// ---- lights (next-event estimation; not in the reference, same expectation) ---------------------------
GBPT_DI uint32_t upper_bound_f(const float* a, uint32_t n, float x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&a[mid]) <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

GBPT_DI float env_pdf(const DevScene& sc, float3 dir) {
    if (sc.ew == 0u) return 0.f;
    const float3 l = normalize(env_to_local(sc, dir));
    const float u = atan2f(l.x, -l.z) * kInv2Pi + 0.5f;
    const float v = acosf(fminf(fmaxf(l.y, -1.f), 1.f)) * kInvPi;
    const float st = sinf(v * kPi);
    if (!(st > 0.f)) return 0.f;
    const int x = min(max((int)floorf(u * sc.ew), 0), (int)sc.ew - 1);
    const int y = min(max((int)floorf(v * sc.eh), 0), (int)sc.eh - 1);
    const float pdf_uv = __ldg(&sc.env_func[(size_t)y * sc.ew + x]) / sc.env_func_int;
    return pdf_uv / (2.0f * kPi * kPi * st);
}

GBPT_DI float tri_light_pdf(const DevScene& sc, float3 le, float dist2, float cos_l) {
    return (1.0f - sc.p_env) * yuv_luminance(le) / sc.light_total * dist2 / fabsf(cos_l);
}

struct LightSample {
    float3 dir, le;
    float dist, pdf;
    bool valid;
};

GBPT_DI LightSample sample_light(const DevScene& sc, float3 pos, Pcg& rng) {
    LightSample ls;
    ls.valid = false;
    const float u0 = rng.next_float(), u1 = rng.next_float(), u2 = rng.next_float();
    if (sc.p_env <= 0.f && sc.n_lights == 0u) return ls;
    if (u0 < sc.p_env) {
        uint32_t y = upper_bound_f(sc.env_marg + 1, sc.eh, u1);
        y = min(y, sc.eh - 1u);
        const float m0 = __ldg(&sc.env_marg[y]), m1 = __ldg(&sc.env_marg[y + 1]);
        const float* c = sc.env_cond + (size_t)y * (sc.ew + 1);
        uint32_t x = upper_bound_f(c + 1, sc.ew, u2);
        x = min(x, sc.ew - 1u);
        const float c0 = __ldg(&c[x]), c1 = __ldg(&c[x + 1]);
        const float fy = fminf(fmaxf((u1 - m0) / (m1 - m0), 0.f), 1.f);
        const float fx = fminf(fmaxf((u2 - c0) / (c1 - c0), 0.f), 1.f);
        const float u = ((float)x + fx) / (float)sc.ew, v = ((float)y + fy) / (float)sc.eh;
        const float phi = kPi * (2.0f * u - 1.0f), theta = kPi * v;
        float sp, cp, st, ct;
        sincosf(phi, &sp, &cp);
        sincosf(theta, &st, &ct);
        const float3 dl = f3(st * sp, ct, -st * cp);
        const float* M = sc.env_m;
        const float3 dw = f3(M[0] * dl.x + M[3] * dl.y + M[6] * dl.z,
                             M[1] * dl.x + M[4] * dl.y + M[7] * dl.z,
                             M[2] * dl.x + M[5] * dl.y + M[8] * dl.z);
        ls.dir = normalize(dw);
        ls.dist = kRayTmax;
        ls.le = env_eval(sc, ls.dir);
        ls.pdf = sc.p_env * env_pdf(sc, ls.dir);
        ls.valid = ls.pdf > 0.f;
        return ls;
    }
    const float ut = sc.p_env > 0.f ? (u0 - sc.p_env) / (1.0f - sc.p_env) : u0;
    uint32_t k = upper_bound_f(sc.light_cdf, sc.n_lights, ut);
    k = min(k, sc.n_lights - 1u);
    const float4 a4 = __ldg(&sc.light_tris[3 * k + 0]);
    const float4 b4 = __ldg(&sc.light_tris[3 * k + 1]);
    const float4 c4 = __ldg(&sc.light_tris[3 * k + 2]);
    const float3 a = f3(a4.x, a4.y, a4.z), b = f3(b4.x, b4.y, b4.z), c = f3(c4.x, c4.y, c4.z);
    const float x = sqrtf(u1);
    const float3 pl = ((1.0f - x) * a + (x * (1.0f - u2)) * b) + (x * u2) * c;
    float3 n = normalize(cross(b - a, c - a));
    if (__float_as_uint(b4.w) & 1u) n = -n;
    const float3 dv = pl - pos;
    const float dist2 = dot(dv, dv);
    const float dist = sqrtf(dist2);
    ls.dir = dv / dist;
    const float cos_l = -dot(ls.dir, n);
    if (!(cos_l > 0.f) || !(dist > 0.f)) return ls;
    const uint32_t mid = sc.geoms[__float_as_uint(a4.w)].material;
    const float4 m2 = __ldg(&sc.mats[5 * mid + 2]);
    ls.le = f3(m2.y, m2.z, m2.w);
    ls.dist = dist * (1.0f - 1e-4f);
    ls.pdf = tri_light_pdf(sc, ls.le, dist2, cos_l);
    ls.valid = ls.pdf > 0.f;
    return ls;
}

// ---- kernels -----------------------------------------------------------------------------------------
struct FrameArgs {
    CamGPU cam;
    uint32_t width, height;
    int spp, max_len;
    int emission_on_primary;
    uint32_t mask;
    uint32_t frame;
    int nee, rr_depth;
    const uint32_t* pixels; // device list or nullptr
    uint32_t pix_base;      // first pixel (list index) of this wave
    uint32_t pix_count;     // pixels in this wave
    Work w;
};

GBPT_DI uint32_t wave_pixel_id(const FrameArgs& a, uint32_t slot) {
    const uint32_t li = a.pix_base + slot;
    return a.pixels ? __ldg(&a.pixels[li]) : li;
}

// Primary hit + shading point per pixel (gbuffer_rt.slang:18-58 + render_pt.slang:98-103)
__global__ void __launch_bounds__(128) k_primary(DevScene sc, FrameArgs a) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= a.pix_count) return;
    const uint32_t pid = wave_pixel_id(a, slot);
    const uint32_t px = pid % a.width, py = pid / a.width;
    float3 o, d;
    float tmin, tmax;
    camera_ray(a.cam, px, py, a.width, a.height, o, d, tmin, tmax);
    const Hit h = trace_ray<false, false>(sc, o, d, tmin, tmax, a.mask, nullptr, a.w.counters + 3);
    SPd sp;
    if (h.geom == 0xFFFFFFFFu || h.geom >= sc.geom_count) {
        sp = env_sp(sc, o, d);
    } else {
        sp = surface_sp(sc, o, d, h.geom, h.prim, round_half(h.u), round_half(h.v));
    }
    float4* pc = a.w.pix + 6ull * slot;
    pc[0] = make_float4(sp.pos.x, sp.pos.y, sp.pos.z, __uint_as_float(sp.enc_fn));
    pc[1] = make_float4(sp.frame.n.x, sp.frame.n.y, sp.frame.n.z, __uint_as_float(sp.mat));
    const uint32_t fl = (sp.has_material ? 1u : 0u) | (sp.front ? 2u : 0u);
    pc[2] = make_float4(sp.frame.t.x, sp.frame.t.y, sp.frame.t.z, __uint_as_float(fl));
    pc[3] = make_float4(sp.frame.b.x, sp.frame.b.y, sp.frame.b.z, 0.f);
    pc[4] = make_float4(sp.emission.x, sp.emission.y, sp.emission.z, 0.f);
    pc[5] = make_float4(d.x, d.y, d.z, 0.f);
    if (slot == 0) atomicAdd(a.w.stats + 0, (unsigned long long)a.pix_count);
}

// Scatter from a shading point (one iteration of the trace_path loop, render_pt.slang:35-79).
// Returns true and the next ray when the path continues; may emit one shadow ray.
template <bool NEE>
GBPT_DI bool scatter(const DevScene& sc, const FrameArgs& a, int k, const SPd& sp, float3 ray_d,
                     float3& thr, float& ior, float3& rad, float& last_pdf, Pcg& rng,
                     float3& no, float3& nd, bool& want_shadow, float4& s_o, float4& s_d,
                     float4& s_c) {
    want_shadow = false;
    if (!sp.has_material || (thr.x < kThroughputMin && thr.y < kThroughputMin && thr.z < kThroughputMin))
        return false;
    if (a.rr_depth > 0 && k >= a.rr_depth) {
        const float q = fminf(1.0f, max3(thr));
        if (rng.next_float() >= q) return false;
        thr = thr / q;
    }
    const Material m = load_material(sc, sp.mat, sp.front, ior);
    const float3 wi_local = sp.frame.to_local(-ray_d);
    const float3 ng = decode_normal(sp.enc_fn);
    const float wi_ng = dot(-ray_d, ng);
    if (NEE) {
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
template <bool NEE>
__global__ void __launch_bounds__(128) k_shade_primary(DevScene sc, FrameArgs a, uint32_t n_paths) {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_round = (n_paths + 31u) & ~31u;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_round; p += stride) {
        bool want = false, want_shadow = false;
        float3 no, nd;
        float4 s_o, s_d, s_c;
        if (p < n_paths) {
            const uint32_t slot = p / (uint32_t)a.spp, s = p % (uint32_t)a.spp;
            const uint32_t pid = wave_pixel_id(a, slot);
            const uint32_t px = pid % a.width, py = pid / a.width;
            Pcg rng{pcg4d16(px, py, a.frame, s)};
            const float4* pc = a.w.pix + 6ull * slot;
            const float4 c0 = pc[0], c1 = pc[1], c2 = pc[2], c3 = pc[3], c4 = pc[4], c5 = pc[5];
            SPd sp;
            sp.pos = f3(c0.x, c0.y, c0.z);
            sp.enc_fn = __float_as_uint(c0.w);
            sp.frame.n = f3(c1.x, c1.y, c1.z);
            sp.mat = __float_as_uint(c1.w);
            sp.frame.t = f3(c2.x, c2.y, c2.z);
            const uint32_t fl = __float_as_uint(c2.w);
            sp.has_material = fl & 1u;
            sp.front = (fl & 2u) != 0u;
            sp.frame.b = f3(c3.x, c3.y, c3.z);
            sp.emission = f3(c4.x, c4.y, c4.z);
            const float3 d = f3(c5.x, c5.y, c5.z);
            float3 thr = f3(1.f, 1.f, 1.f);
            float ior = 1.0f;
            float3 rad = a.emission_on_primary ? sp.emission : f3(0.f, 0.f, 0.f);
            float last_pdf = 0.f;
            if (a.max_len > 1)
                want = scatter<NEE>(sc, a, 1, sp, d, thr, ior, rad, last_pdf, rng, no, nd,
                                    want_shadow, s_o, s_d, s_c);
            a.w.thr[p] = make_float4(thr.x, thr.y, thr.z, ior);
            a.w.rad[p] = make_float4(rad.x, rad.y, rad.z, last_pdf);
            a.w.rng[p] = rng.state;
        }
        const uint32_t q = warp_append(a.w.counters + 0, want);
        if (want) {
            a.w.q_od[0][2 * q + 0] = make_float4(no.x, no.y, no.z, 0.f);
            a.w.q_od[0][2 * q + 1] = make_float4(nd.x, nd.y, nd.z, kRayTmax);
            a.w.q_path[0][q] = p;
        }
        if (NEE) {
            const uint32_t sq = warp_append(a.w.counters + 2, want_shadow);
            if (want_shadow) {
                a.w.s_od[2 * sq + 0] = s_o;
                a.w.s_od[2 * sq + 1] = s_d;
                a.w.s_contrib[sq] = s_c;
                a.w.s_path[sq] = p;
            }
        }
    }
}

// Resident 128-thread blocks per SM the traversal kernels are register-budgeted for
// (65536 / (8 * 128) = 64 registers per thread).
constexpr int kTraceBlocksPerSM = 8;

// Closest hit for every entry of ray queue `qi` (persistent warps, counter w.counters[4]).
template <bool COUNT>
__global__ void __launch_bounds__(128, kTraceBlocksPerSM) k_trace(DevScene sc, Work w, int qi, uint32_t mask,
                                               unsigned long long* work_ctr) {
    const uint32_t n = w.counters[qi];
    TraceCounters ctr{0, 0};
    const float4* q = w.q_od[qi];
    auto load = [&](uint32_t i, float3& o, float3& d, float& tmin, float& tmax) {
        const float4 a = q[2 * i + 0];
        const float4 b = q[2 * i + 1];
        o = f3(a.x, a.y, a.z);
        d = f3(b.x, b.y, b.z);
        tmin = a.w;
        tmax = b.w;
    };
    auto store = [&](uint32_t i, const Hit& h) {
        w.hit_tuv[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        w.hit_geom[i] = h.geom;
    };
    trace_persistent<false, COUNT>(sc, n, w.counters + 4, mask, load, store, &ctr, w.counters + 3);
    if (COUNT) {
        atomicAdd(work_ctr + 0, (unsigned long long)ctr.nodes);
        atomicAdd(work_ctr + 1, (unsigned long long)ctr.tris);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(w.stats + 0, (unsigned long long)n);
        atomicAdd(w.stats + 2, (unsigned long long)n);
    }
}

// Emission at the k-th path vertex, then scatter (k < L) into ray queue `qo`.
template <bool NEE>
__global__ void __launch_bounds__(128) k_shade(DevScene sc, FrameArgs a, int k, int qi, int qo) {
    const uint32_t n = a.w.counters[qi];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_round = (n + 31u) & ~31u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        bool want = false, want_shadow = false;
        float3 no, nd;
        float4 s_o, s_d, s_c;
        uint32_t p = 0;
        if (i < n) {
            p = a.w.q_path[qi][i];
            const float4 qa = a.w.q_od[qi][2 * i + 0];
            const float4 qb = a.w.q_od[qi][2 * i + 1];
            const float3 o = f3(qa.x, qa.y, qa.z), d = f3(qb.x, qb.y, qb.z);
            const float4 h = a.w.hit_tuv[i];
            const uint32_t geom = a.w.hit_geom[i];
            const float4 t4 = a.w.thr[p], r4 = a.w.rad[p];
            float3 thr = f3(t4.x, t4.y, t4.z), rad = f3(r4.x, r4.y, r4.z);
            float ior = t4.w, last_pdf = r4.w;
            Pcg rng{a.w.rng[p]};
            SPd sp;
            if (geom == 0xFFFFFFFFu || geom >= sc.geom_count) {
                sp = env_sp(sc, o, d);
            } else {
                sp = surface_sp(sc, o, d, geom, __float_as_uint(h.w), h.y, h.z);
            }
            sp.has_material = sp.has_material && (k < a.max_len);
            float3 e = thr * sp.emission;
            if (NEE && !all_zero(e)) {
                float pl = 0.f;
                if (sp.env) pl = sc.p_env * env_pdf(sc, d);
                else if (sp.emissive) pl = tri_light_pdf(sc, sp.emission, h.x * h.x, dot(d, sp.fn));
                e = e * power_heuristic(last_pdf, pl);
            }
            rad = rad + e;
            if (k < a.max_len)
                want = scatter<NEE>(sc, a, k, sp, d, thr, ior, rad, last_pdf, rng, no, nd,
                                    want_shadow, s_o, s_d, s_c);
            a.w.thr[p] = make_float4(thr.x, thr.y, thr.z, ior);
            a.w.rad[p] = make_float4(rad.x, rad.y, rad.z, last_pdf);
            a.w.rng[p] = rng.state;
        }
        const uint32_t q = warp_append(a.w.counters + qo, want);
        if (want) {
            a.w.q_od[qo][2 * q + 0] = make_float4(no.x, no.y, no.z, 0.f);
            a.w.q_od[qo][2 * q + 1] = make_float4(nd.x, nd.y, nd.z, kRayTmax);
            a.w.q_path[qo][q] = p;
        }
        if (NEE) {
            const uint32_t sq = warp_append(a.w.counters + 2, want_shadow);
            if (want_shadow) {
                a.w.s_od[2 * sq + 0] = s_o;
                a.w.s_od[2 * sq + 1] = s_d;
                a.w.s_contrib[sq] = s_c;
                a.w.s_path[sq] = p;
            }
        }
    }
}

// Occlusion of the NEE queue; unoccluded contributions are added to their path.
__global__ void __launch_bounds__(128, kTraceBlocksPerSM) k_shadow(DevScene sc, Work w, uint32_t mask) {
    const uint32_t n = w.counters[2];
    auto load = [&](uint32_t i, float3& o, float3& d, float& tmin, float& tmax) {
        const float4 a = w.s_od[2 * i + 0];
        const float4 b = w.s_od[2 * i + 1];
        o = f3(a.x, a.y, a.z);
        d = f3(b.x, b.y, b.z);
        tmin = 0.0f;
        tmax = a.w;
    };
    auto store = [&](uint32_t i, const Hit& h) {
        if (h.geom == 0xFFFFFFFFu) {
            const uint32_t p = w.s_path[i];
            const float4 c = w.s_contrib[i];
            float4 r = w.rad[p];
            r.x += c.x;
            r.y += c.y;
            r.z += c.z;
            w.rad[p] = r;
        }
    };
    trace_persistent<true, false>(sc, n, w.counters + 5, mask, load, store, nullptr,
                                  w.counters + 3);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(w.stats + 0, (unsigned long long)n);
        atomicAdd(w.stats + 1, (unsigned long long)n);
    }
}

// Per-pixel mean and mean squared luminance over the samples (render_pt.slang:110-129); one warp
// per pixel, lanes stride the samples, fixed shuffle tree: a deterministic summation order.
__global__ void __launch_bounds__(128) k_finalize(FrameArgs a, float4* out, uint32_t out_base) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (warp >= a.pix_count) return;
    const uint32_t S = (uint32_t)a.spp;
    float r = 0.f, g = 0.f, b = 0.f, m = 0.f;
    for (uint32_t s = lane; s < S; s += 32u) {
        const float4 c = a.w.rad[(size_t)warp * S + s];
        if (isfinite(c.x) && isfinite(c.y) && isfinite(c.z)) {
            r += c.x;
            g += c.y;
            b += c.z;
            const float l = yuv_luminance(f3(c.x, c.y, c.z));
            m += l * l;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        r += __shfl_xor_sync(0xFFFFFFFFu, r, off);
        g += __shfl_xor_sync(0xFFFFFFFFu, g, off);
        b += __shfl_xor_sync(0xFFFFFFFFu, b, off);
        m += __shfl_xor_sync(0xFFFFFFFFu, m, off);
    }
    if (lane == 0) {
        const float inv = S > 0 ? 1.0f / (float)S : 0.f;
        out[out_base + warp] = make_float4(r * inv, g * inv, b * inv, m * inv);
    }
}

template <bool ANY>
__global__ void __launch_bounds__(128, kTraceBlocksPerSM) k_trace_rays(DevScene sc, const gbpt_ray* rays, uint32_t n,
                                                    uint32_t mask, gbpt_hit* hits,
                                                    unsigned long long* work_ctr, uint32_t* fetch,
                                                    uint32_t* err) {
    TraceCounters ctr{0, 0};
    auto load = [&](uint32_t i, float3& o, float3& d, float& tmin, float& tmax) {
        const gbpt_ray r = rays[i];
        o = f3(r.origin[0], r.origin[1], r.origin[2]);
        d = f3(r.direction[0], r.direction[1], r.direction[2]);
        tmin = r.tmin;
        tmax = r.tmax;
    };
    auto store = [&](uint32_t i, const Hit& h) {
        gbpt_hit out;
        const bool ok = h.geom != 0xFFFFFFFFu;
        out.instance_id = ok ? 0u : 0xFFFFFFFFu;
        out.instance_index = ok ? 0u : 0xFFFFFFFFu;
        out.primitive_id = h.prim;
        out.geometry_index = h.geom;
        out.barycentrics[0] = ok ? h.u : 0.f;
        out.barycentrics[1] = ok ? h.v : 0.f;
        out.t = ok ? h.t : -1.0f;
        out.reserved = 0;
        hits[i] = out;
    };
    trace_persistent<ANY, true>(sc, n, fetch, mask, load, store, &ctr, err);
    if (work_ctr) {
        atomicAdd(work_ctr + 0, (unsigned long long)ctr.nodes);
        atomicAdd(work_ctr + 1, (unsigned long long)ctr.tris);
    }
}

__global__ void k_trace_primary(DevScene sc, CamGPU cam, uint32_t w, uint32_t h, uint32_t mask,
                                gbpt_hit* hits, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    float3 o, d;
    float tmin, tmax;
    camera_ray(cam, i % w, i / w, w, h, o, d, tmin, tmax);
    const Hit ht = trace_ray<false, false>(sc, o, d, tmin, tmax, mask, nullptr, err);
    gbpt_hit out;
    const bool ok = ht.geom != 0xFFFFFFFFu;
    out.instance_id = ok ? 0u : 0xFFFFFFFFu;
    out.instance_index = ok ? 0u : 0xFFFFFFFFu;
    out.primitive_id = ht.prim;
    out.geometry_index = ht.geom;
    out.barycentrics[0] = ok ? ht.u : 0.f;
    out.barycentrics[1] = ok ? ht.v : 0.f;
    out.t = ok ? ht.t : -1.0f;
    out.reserved = 0;
    hits[i] = out;
}

// Blocks of 128 threads that fit the whole GPU at once (persistent kernels).
template <class K> int persistent_grid(K kernel) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, 128, 0) != cudaSuccess || nb <= 0)
        nb = 4;
    return nb * num_sms();
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

template <class T> cudaError_t alloc(T*& p, uint64_t n, uint64_t& bytes) {
    bytes += n * sizeof(T);
    return cudaMalloc((void**)&p, n * sizeof(T) + 16);
}

} // namespace

void work_free(Work& w) {
    void* ptrs[] = {w.thr, w.rad, w.rng, w.q_od[0], w.q_od[1], w.q_path[0], w.q_path[1],
                    w.hit_tuv, w.hit_geom, w.s_od, w.s_contrib, w.s_path, w.pix, w.pix_id,
                    w.out, w.counters, w.stats};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    w = Work{};
}

int work_reserve(Work& w, uint64_t paths, uint64_t pixels) {
    if (w.fixed) return (paths <= w.path_cap && pixels <= w.pixel_cap) ? GBPT_OK : GBPT_ERR_NO_MEMORY;
    if (!w.counters) {
        uint64_t b = 0;
        if (alloc(w.counters, 16, b) != cudaSuccess) return GBPT_ERR_NO_MEMORY;
        if (alloc(w.stats, 8, b) != cudaSuccess) return GBPT_ERR_NO_MEMORY;
        cudaMemset(w.counters, 0, 16 * sizeof(uint32_t));
        cudaMemset(w.stats, 0, 8 * sizeof(unsigned long long));
        w.bytes += b;
    }
    if (paths > w.path_cap) {
        void* old[] = {w.thr, w.rad, w.rng, w.q_od[0], w.q_od[1], w.q_path[0], w.q_path[1],
                       w.hit_tuv, w.hit_geom, w.s_od, w.s_contrib, w.s_path};
        for (void* p : old)
            if (p) cudaFree(p);
        uint64_t b = 0;
        bool ok = alloc(w.thr, paths, b) == cudaSuccess && alloc(w.rad, paths, b) == cudaSuccess &&
                  alloc(w.rng, paths, b) == cudaSuccess &&
                  alloc(w.q_od[0], 2 * paths, b) == cudaSuccess &&
                  alloc(w.q_od[1], 2 * paths, b) == cudaSuccess &&
                  alloc(w.q_path[0], paths, b) == cudaSuccess &&
                  alloc(w.q_path[1], paths, b) == cudaSuccess &&
                  alloc(w.hit_tuv, paths, b) == cudaSuccess &&
                  alloc(w.hit_geom, paths, b) == cudaSuccess &&
                  alloc(w.s_od, 2 * paths, b) == cudaSuccess &&
                  alloc(w.s_contrib, paths, b) == cudaSuccess &&
                  alloc(w.s_path, paths, b) == cudaSuccess;
        if (!ok) {
            w.path_cap = 0;
            return GBPT_ERR_NO_MEMORY;
        }
        w.path_cap = paths;
        w.bytes += b;
    }
    if (pixels > w.pixel_cap) {
        if (w.pix) cudaFree(w.pix);
        uint64_t b = 0;
        if (alloc(w.pix, 6 * pixels, b) != cudaSuccess) return GBPT_ERR_NO_MEMORY;
        w.pixel_cap = pixels;
        w.bytes += b;
    }
    return GBPT_OK;
}

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

int render_frame(const SceneGPU& scene, Work& w, const RenderArgs& args, cudaStream_t st,
                 uint64_t* launches, Profile* prof, unsigned long long* work_ctr) {
    Profile dummy;
    if (!prof) prof = &dummy;
    const bool count_work = prof->level >= 2 && work_ctr != nullptr;
    const gbpt_render_params& p = args.params;
    const uint32_t S = (uint32_t)p.spp;
    const uint32_t P = args.pixel_count;
    if (S == 0 || P == 0) return GBPT_OK;
    // wave: whole pixels, as many as fit the wave size (at least one pixel's samples)
    const uint64_t target_paths = std::max<uint64_t>(S, w.fixed ? w.path_cap : kWavePaths);
    const uint32_t pix_per_wave =
        (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(P, target_paths / S));
    int rc = work_reserve(w, (uint64_t)pix_per_wave * S, pix_per_wave);
    if (rc != GBPT_OK) return rc;
    const DevScene sc = make_dev_scene(scene);
    FrameArgs a{};
    a.cam = to_cam(args.camera);
    a.width = p.width;
    a.height = p.height;
    a.spp = p.spp;
    a.max_len = p.max_path_length;
    a.emission_on_primary = p.emission_on_primary;
    a.mask = p.instance_mask & 0xFFu;
    a.frame = p.frame;
    a.nee = p.nee && (scene.n_lights > 0 || scene.env != nullptr);
    a.rr_depth = p.rr_depth;
    a.pixels = args.pixels_device;
    a.w = w;
    const int grid = num_sms() * 8;
    // persistent traversal kernels: exactly the resident blocks
    const int trace_grid = persistent_grid(k_trace<false>);
    const int trace_grid_c = persistent_grid(k_trace<true>);
    const int shadow_grid = persistent_grid(k_shadow);
    uint64_t nl = 0;
    for (uint32_t base = 0; base < P; base += pix_per_wave) {
        a.pix_base = base;
        a.pix_count = std::min(pix_per_wave, P - base);
        const uint32_t n_paths = a.pix_count * S;
        cudaMemsetAsync(w.counters, 0, 3 * sizeof(uint32_t), st);
        int ev = prof->begin(st, 3);
        k_primary<<<(a.pix_count + 127) / 128, 128, 0, st>>>(sc, a);
        prof->end(st, ev);
        const int pgrid = (int)std::min<uint64_t>((n_paths + 127) / 128, (uint64_t)grid);
        ev = prof->begin(st, 1);
        if (a.nee) k_shade_primary<true><<<pgrid, 128, 0, st>>>(sc, a, n_paths);
        else k_shade_primary<false><<<pgrid, 128, 0, st>>>(sc, a, n_paths);
        prof->end(st, ev);
        nl += 2;
        if (a.nee) {
            cudaMemsetAsync(w.counters + 5, 0, sizeof(uint32_t), st);
            ev = prof->begin(st, 2);
            k_shadow<<<shadow_grid, 128, 0, st>>>(sc, w, a.mask);
            prof->end(st, ev);
            cudaMemsetAsync(w.counters + 2, 0, sizeof(uint32_t), st);
            nl += 1;
        }
        int qi = 0;
        for (int k = 2; k <= a.max_len; ++k) {
            const int qo = qi ^ 1;
            cudaMemsetAsync(w.counters + 4, 0, sizeof(uint32_t), st);
            ev = prof->begin(st, 0);
            if (count_work) k_trace<true><<<trace_grid_c, 128, 0, st>>>(sc, w, qi, a.mask, work_ctr);
            else k_trace<false><<<trace_grid, 128, 0, st>>>(sc, w, qi, a.mask, nullptr);
            prof->end(st, ev);
            cudaMemsetAsync(w.counters + qo, 0, sizeof(uint32_t), st);
            ev = prof->begin(st, 1);
            if (a.nee) k_shade<true><<<grid, 128, 0, st>>>(sc, a, k, qi, qo);
            else k_shade<false><<<grid, 128, 0, st>>>(sc, a, k, qi, qo);
            prof->end(st, ev);
            nl += 2;
            if (a.nee && k < a.max_len) {
                cudaMemsetAsync(w.counters + 5, 0, sizeof(uint32_t), st);
                ev = prof->begin(st, 2);
                k_shadow<<<shadow_grid, 128, 0, st>>>(sc, w, a.mask);
                prof->end(st, ev);
                cudaMemsetAsync(w.counters + 2, 0, sizeof(uint32_t), st);
                nl += 1;
            }
            qi = qo;
        }
        const uint32_t fin_threads = a.pix_count * 32u;
        ev = prof->begin(st, 3);
        k_finalize<<<(fin_threads + 127) / 128, 128, 0, st>>>(a, args.out_device, base);
        prof->end(st, ev);
        nl += 1;
    }
    if (launches) *launches += nl;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return GBPT_ERR_CUDA;
    return GBPT_OK;
}

int primary_points(const SceneGPU& scene, Work& w, const RenderArgs& args, cudaStream_t st,
                   float* out_device) {
    const uint32_t P = args.pixel_count;
    int rc = work_reserve(w, std::max<uint64_t>(P, 1), std::max<uint64_t>(P, 1));
    if (rc != GBPT_OK) return rc;
    FrameArgs a{};
    a.cam = to_cam(args.camera);
    a.width = args.params.width;
    a.height = args.params.height;
    a.mask = args.params.instance_mask & 0xFFu;
    a.pixels = args.pixels_device;
    a.pix_base = 0;
    a.pix_count = P;
    a.w = w;
    k_primary<<<(P + 127) / 128, 128, 0, st>>>(make_dev_scene(scene), a);
    if (cudaMemcpyAsync(out_device, w.pix, (size_t)P * 6 * sizeof(float4), cudaMemcpyDeviceToDevice,
                        st) != cudaSuccess)
        return GBPT_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? GBPT_OK : GBPT_ERR_CUDA;
}

int trace_rays(const SceneGPU& scene, const gbpt_ray* rays, uint32_t n, uint32_t mask, int any_hit,
               gbpt_hit* hits, unsigned long long* work_ctr, cudaStream_t st) {
    if (n == 0) return GBPT_OK;
    const DevScene sc = make_dev_scene(scene);
    uint32_t* err = reinterpret_cast<uint32_t*>(work_ctr + 2);
    uint32_t* fetch = reinterpret_cast<uint32_t*>(work_ctr + 3);
    cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st);
    if (any_hit)
        k_trace_rays<true><<<persistent_grid(k_trace_rays<true>), 128, 0, st>>>(
            sc, rays, n, mask & 0xFFu, hits, work_ctr, fetch, err);
    else
        k_trace_rays<false><<<persistent_grid(k_trace_rays<false>), 128, 0, st>>>(
            sc, rays, n, mask & 0xFFu, hits, work_ctr, fetch, err);
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
// per path: throughput, radiance (16 + 16), rng (4), two ray queues (2 x 36), hits (20),
// shadow queue (52); plus a 96-byte primary point per pixel, budgeted as one pixel per path
constexpr uint64_t kStaticBytesPerPath = 16 + 16 + 4 + 2 * (32 + 4) + (16 + 4) + (32 + 16 + 4) + 96;

std::mutex g_static_mu;
void* g_static_ptr[64] = {};

// The array's device address on the current device, looked up on the first call per device.
int static_scratch_address(int dev, unsigned char** out) {
    if (dev < 0 || dev >= 64) return GBPT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) return GBPT_ERR_CUDA;
        g_static_ptr[dev] = p;
    }
    *out = (unsigned char*)g_static_ptr[dev];
    return GBPT_OK;
}
} // namespace

uint64_t static_scratch_paths() {
    // 16 x 256 bytes of slack for the alignment of the carved arrays
    return (kStaticScratchBytes - kStaticCounterBytes - kStaticPixelBytes - 16 * 256) /
           kStaticBytesPerPath;
}

int render_frame_static(const SceneGPU& scene, const RenderArgs& args, const uint32_t* pixels_host,
                        cudaStream_t st, std::string& err) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        err = "cudaGetDevice failed";
        return GBPT_ERR_CUDA;
    }
    unsigned char* base = nullptr;
    int rc = static_scratch_address(dev, &base);
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
    // carve the work buffers: counters, pixel list, then per-path and per-pixel arrays
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
    carve(w.thr, N);
    carve(w.rad, N);
    carve(w.rng, N);
    carve(w.q_od[0], 2 * N);
    carve(w.q_od[1], 2 * N);
    carve(w.q_path[0], N);
    carve(w.q_path[1], N);
    carve(w.hit_tuv, N);
    carve(w.hit_geom, N);
    carve(w.s_od, 2 * N);
    carve(w.s_contrib, N);
    carve(w.s_path, N);
    carve(w.pix, 6 * N);
    if ((uint64_t)(p - base) > kStaticScratchBytes) {
        err = "static scratch layout overflow";
        return GBPT_ERR_INVALID;
    }
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

int trace_primary(const SceneGPU& scene, const gbpt_camera& cam, uint32_t w, uint32_t h,
                  uint32_t mask, gbpt_hit* hits, uint32_t* err, cudaStream_t st) {
    const DevScene sc = make_dev_scene(scene);
    const uint32_t n = w * h;
    k_trace_primary<<<(n + 127) / 128, 128, 0, st>>>(sc, to_cam(cam), w, h, mask & 0xFFu, hits, err);
    return cudaGetLastError() == cudaSuccess ? GBPT_OK : GBPT_ERR_CUDA;
}

} // namespace gbpt

// Shading points, material instances and light sampling for the wavefront kernels.
#pragma once

#include "device_scene.cuh"
#include "runtime.h"

namespace gbpt {

// Device view of a resident scene.
inline DevScene make_dev_scene(const SceneGPU& s) {
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

// Appends one entry per lane that wants one; one atomic per warp. All 32 lanes must call it.
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

// _make_environment_map_shading_point (scene.slang:482-498)
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

// get_triangle_hit + get_surface + get_shading_point (scene.slang:312-456), material instantiated
// later by the scatter step
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

// solid-angle density of the environment strategy (piecewise constant over texels)
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

// solid-angle density of reaching an emissive triangle point: selection by power (area x
// luminance), uniform area sampling; the area cancels
GBPT_DI float tri_light_pdf(const DevScene& sc, float3 le, float dist2, float cos_l) {
    return (1.0f - sc.p_env) * yuv_luminance(le) / sc.light_total * dist2 / fabsf(cos_l);
}

struct LightSample {
    float3 dir, le;
    float dist, pdf;
    bool valid;
};

// Three draws: strategy/triangle choice, then two for the point (sample_triangle,
// utils/sampling.slang:31-36) or the environment texel (marginal row, conditional column).
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

// Blocks of 128 threads that fit the whole GPU at once (persistent kernels).
int num_sms();
template <class K> int persistent_grid(K kernel) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, 128, 0) != cudaSuccess || nb <= 0)
        nb = 4;
    return nb * num_sms();
}

// Resident 128-thread blocks per SM the traversal kernels are register-budgeted for
// (65536 / (8 * 128) = 64 registers per thread).
#ifndef GBPT_TRACE_BLOCKS_PER_SM
#define GBPT_TRACE_BLOCKS_PER_SM 8
#endif
constexpr int kTraceBlocksPerSM = GBPT_TRACE_BLOCKS_PER_SM;

} // namespace gbpt

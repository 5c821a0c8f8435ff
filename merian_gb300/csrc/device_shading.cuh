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
    d.tri_stride = (uint32_t)(3u * s.n_tris);
    d.verts = (const uint32_t*)s.verts;
    d.idx = (const uint32_t*)s.idx;
    d.tri_verts = (const uint4*)s.tri_verts;
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
    d.light_guide = (const uint32_t*)s.light_guide;
    d.env_rows = (const uint2*)s.env_rows;
    d.env_cols = (const uint2*)s.env_cols;
    d.env_marg_guide = (const uint32_t*)s.env_marg_guide;
    d.env_cond_guide = (const uint32_t*)s.env_cond_guide;
    d.light_g = s.light_g;
    d.env_marg_g = s.env_marg_g;
    d.env_cond_g = s.env_cond_g;
    d.p_env = d.ew ? (s.n_lights ? 0.5f : 1.0f) : 0.0f;
    d.inst = (const float4*)s.inst;
    d.n_inst = s.n_inst;
    d.tex = (const uchar4*)s.tex;
    d.tex_info = (const uint4*)s.tex_info;
    d.n_tex = s.n_tex;
    d.srgb_lut = (const float*)s.srgb_lut;
    return d;
}

// Bilinear lookup with repeat addressing at level 0 (merian's DefaultLODSampler = LOD0Sampler,
// textures.slang:338-423, on a linear/repeat sampler): texel centres at (i + 0.5) / size; an sRGB
// texture is decoded per texel before filtering, as the hardware does for sRGB formats.
GBPT_DI float4 texture_sample(const DevScene& sc, uint32_t t, float u, float v) {
    const uint4 info = __ldg(&sc.tex_info[t]);
    const int w = (int)info.y, h = (int)info.z;
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    const int ix = (int)fx, iy = (int)fy;
    const int x0 = ((ix % w) + w) % w, x1 = (((ix + 1) % w) + w) % w;
    const int y0 = ((iy % h) + h) % h, y1 = (((iy + 1) % h) + h) % h;
    const uchar4* base = sc.tex + info.x;
    auto texel = [&](int xx, int yy) {
        const uchar4 c = __ldg(&base[(size_t)yy * w + xx]);
        if (info.w)
            return make_float4(__ldg(&sc.srgb_lut[c.x]), __ldg(&sc.srgb_lut[c.y]),
                               __ldg(&sc.srgb_lut[c.z]), (float)c.w * (1.0f / 255.0f));
        return make_float4((float)c.x * (1.0f / 255.0f), (float)c.y * (1.0f / 255.0f),
                           (float)c.z * (1.0f / 255.0f), (float)c.w * (1.0f / 255.0f));
    };
    const float4 t00 = texel(x0, y0), t10 = texel(x1, y0), t01 = texel(x0, y1), t11 = texel(x1, y1);
    auto mix = [&](float c00, float c10, float c01, float c11) {
        const float top = c00 * (1.0f - a) + c10 * a;
        const float bot = c01 * (1.0f - a) + c11 * a;
        return top * (1.0f - b) + bot * b;
    };
    return make_float4(mix(t00.x, t10.x, t01.x, t11.x), mix(t00.y, t10.y, t01.y, t11.y),
                       mix(t00.z, t10.z, t01.z, t11.z), mix(t00.w, t10.w, t01.w, t11.w));
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
    float3 tex_color; // base colour texture at the hit (1 without a texture)
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
// the environment seen along d, its map coordinates (u, v) already known
GBPT_DI SPd env_sp_uv(const DevScene& sc, float3 o, float3 d, float u, float v) {
    SPd sp;
    sp.pos = o + d * kEnvDistance;
    sp.enc_fn = encode_normal(-d);
    sp.fn = -d;
    sp.emission = sc.ew ? env_eval_uv(sc, u, v) : f3(0.f, 0.f, 0.f);
    sp.frame = frame_from_normal(-d);
    sp.tex_color = f3(1.f, 1.f, 1.f);
    sp.mat = 0;
    sp.has_material = false;
    sp.front = true;
    sp.emissive = false;
    sp.env = true;
    return sp;
}
GBPT_DI SPd env_sp(const DevScene& sc, float3 o, float3 d) {
    float u = 0.f, v = 0.f;
    if (sc.ew) env_uv(sc, d, u, v);
    return env_sp_uv(sc, o, d, u, v);
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
// A two-level hit (inst != kNoInst) is transformed to world space as scene.slang:235-259 does:
// position by the object-to-world transform, edges and tangents by its linear part, the
// interpolated normal by the inverse transpose (renormalised).
GBPT_DI SPd surface_sp(const DevScene& sc, float3 o, float3 d, uint32_t geom, uint32_t prim,
                       float bu, float bv, uint32_t inst = kNoInst) {
    const GeomGPU g = sc.geoms[geom];
    if (g.flags & GBPT_MESH_USE_ENV_MAP) return env_sp(sc, o, d);
    const uint32_t tri = g.first_triangle + prim;
    float3 p0, p1, p2;
    uint32_t n0, n1, n2, uv0, uv1, uv2, t0, t1, t2;
    if (sc.tri_verts) { // the triangle's record: no index fetch before the vertex loads
        const uint4* r = sc.tri_verts + 5ull * tri;
        const uint4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), e = __ldg(r + 3),
                    f = __ldg(r + 4);
        p0 = f3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
        n0 = a.w, uv0 = b.x, t0 = b.y;
        p1 = f3(__uint_as_float(b.z), __uint_as_float(b.w), __uint_as_float(c.x));
        n1 = c.y, uv1 = c.z, t1 = c.w;
        p2 = f3(__uint_as_float(e.x), __uint_as_float(e.y), __uint_as_float(e.z));
        n2 = e.w, uv2 = f.x, t2 = f.y;
    } else {
        load_vertex(sc, g.first_vertex + __ldg(&sc.idx[3 * tri + 0]), p0, n0, uv0, t0);
        load_vertex(sc, g.first_vertex + __ldg(&sc.idx[3 * tri + 1]), p1, n1, uv1, t1);
        load_vertex(sc, g.first_vertex + __ldg(&sc.idx[3 * tri + 2]), p2, n2, uv2, t2);
    }
    const float b0 = 1.0f - bu - bv, b1 = bu, b2 = bv;
    const bool xf = inst != kNoInst;
    float4 x0, x1, x2, w0r, w1r, w2r;
    if (xf) {
        const float4* r = sc.inst + 7ull * inst;
        x0 = __ldg(r + 0);
        x1 = __ldg(r + 1);
        x2 = __ldg(r + 2);
        w0r = __ldg(r + 3);
        w1r = __ldg(r + 4);
        w2r = __ldg(r + 5);
    }
    float3 pos = (b0 * p0 + b1 * p1) + b2 * p2;
    float3 e01 = p1 - p0, e02 = p2 - p0;
    if (xf) {
        pos = xform_point(x0, x1, x2, pos);
        e01 = xform_vector(x0, x1, x2, e01);
        e02 = xform_vector(x0, x1, x2, e02);
    }
    float3 fn = normalize(cross(e01, e02));
    if (g.flags & GBPT_MESH_FLIP_FACING) fn = -fn;
    float3 vn;
    if (g.flags & GBPT_MESH_FLAT_SHADING) {
        vn = fn;
    } else {
        vn = normalize((b0 * decode_normal(n0) + b1 * decode_normal(n1)) + b2 * decode_normal(n2));
        if (xf) { // inverse transpose: the columns of the world-to-object rows
            vn = normalize(f3(w0r.x * vn.x + w1r.x * vn.y + w2r.x * vn.z,
                              w0r.y * vn.x + w1r.y * vn.y + w2r.y * vn.z,
                              w0r.z * vn.x + w1r.z * vn.y + w2r.z * vn.z));
        }
    }
    Frame frame;
    if (g.flags & GBPT_MESH_HAS_TANGENTS) {
        const float w0 = (t0 & 1u) ? -1.f : 1.f, w1 = (t1 & 1u) ? -1.f : 1.f,
                    w2 = (t2 & 1u) ? -1.f : 1.f;
        const float3 t = (b0 * decode_normal(t0 & ~1u) + b1 * decode_normal(t1 & ~1u)) +
                         b2 * decode_normal(t2 & ~1u);
        const float tw = (b0 * w0 + b1 * w1) + b2 * w2;
        float3 tn = normalize(t);
        if (xf) tn = xform_vector(x0, x1, x2, tn);
        frame = frame_from_tangent(vn, tn, signf(tw));
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
    sp.tex_color = f3(1.f, 1.f, 1.f);
    if (sc.n_tex) { // the base colour texture (the material header's alpha texture)
        const int tex = (int)__float_as_uint(__ldg(&sc.mats[5 * g.material + 4]).x);
        if (tex >= 0 && (uint32_t)tex < sc.n_tex) {
            const float u = (b0 * half_lo(uv0) + b1 * half_lo(uv1)) + b2 * half_lo(uv2);
            const float v = (b0 * half_hi(uv0) + b1 * half_hi(uv1)) + b2 * half_hi(uv2);
            const float4 c = texture_sample(sc, (uint32_t)tex, u, v);
            sp.tex_color = f3(c.x, c.y, c.z);
        }
    }
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
// tex: the base colour texture at the shading point, multiplying base_color
// (diffuse-material.slang:25-29, openpbr-material.slang:114-116)
GBPT_DI Material load_material(const DevScene& sc, uint32_t mid, bool front, float ior,
                               float3 tex = f3(1.f, 1.f, 1.f)) {
    Material m = material_from_record(__ldg(&sc.mats[5 * mid + 0]), __ldg(&sc.mats[5 * mid + 1]),
                                      __ldg(&sc.mats[5 * mid + 2]), __ldg(&sc.mats[5 * mid + 3]),
                                      front, ior);
    m.base = m.base * tex;
    return m;
}

// ---- lights (next-event estimation; not in the reference, same expectation) ---------------------------
// upper_bound(a, a + n, x) for x in [0, 1), the search narrowed by the CDF's guide table g (G
// entries + 1): x * G is exact for a power-of-two G, so the bound lies in [g[k], g[k + 1]].
GBPT_DI uint32_t upper_bound_f(const float* a, uint32_t n, float x, const uint32_t* g, uint32_t G) {
    uint32_t lo = 0, hi = n;
    if (G) {
        const uint32_t k = min((uint32_t)(x * (float)G), G - 1u);
        lo = __ldg(&g[k]);
        hi = __ldg(&g[k + 1]);
    }
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&a[mid]) <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Bin (k n) >> 24 of n for the draw u = k 2^-24, and the rest of k n as a fraction in [0, 1):
// a uniform choice of the bin and, independent of it, a uniform fraction.
GBPT_DI uint32_t bin_of(float u, uint32_t n, float& frac) {
    const uint64_t kn = (uint64_t)(uint32_t)(u * 16777216.0f) * n;
    frac = (float)(uint32_t)(kn & 0xFFFFFFull) * 5.9604644775390625e-08f;
    return (uint32_t)(kn >> 24);
}

// Bin i of the alias table t (Walker 1977) keeps i when the uniform d is below its keep
// probability and gives its alias otherwise; d is rescaled to [0, 1) within the branch taken, a
// uniform independent of the outcome, for the next decision.
GBPT_DI uint32_t alias_pick(const uint2* t, uint32_t i, float& d) {
    const uint2 e = __ldg(&t[i]);
    const float p = __uint_as_float(e.x);
    if (d < p) {
        d = d / p;
        return i;
    }
    d = (d - p) / (1.0f - p);
    return e.y;
}

// solid-angle density of the environment strategy (piecewise constant over texels)
// the density at map point (u, v) given sin(pi v)
GBPT_DI float env_pdf_st(const DevScene& sc, float u, float v, float st) {
    if (!(st > 0.f)) return 0.f;
    const int x = min(max((int)floorf(u * sc.ew), 0), (int)sc.ew - 1);
    const int y = min(max((int)floorf(v * sc.eh), 0), (int)sc.eh - 1);
    const float pdf_uv = __ldg(&sc.env_func[(size_t)y * sc.ew + x]) / sc.env_func_int;
    return pdf_uv / (2.0f * kPi * kPi * st);
}
GBPT_DI float env_pdf_uv(const DevScene& sc, float u, float v) {
    return env_pdf_st(sc, u, v, sinf(v * kPi));
}
GBPT_DI float env_pdf(const DevScene& sc, float3 dir) {
    if (sc.ew == 0u) return 0.f;
    float u, v;
    env_uv(sc, dir, u, v);
    return env_pdf_uv(sc, u, v);
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
#if GBPT_ENV_ALIAS
        // the row by the row table, then the column by that row's table: u1 and u2 choose the
        // bins and, by their fractions, the point in the texel; the strategy draw, rescaled
        // (p_env is 1 or 1/2, so exactly), makes both keep-or-alias decisions
        float d = u0 / sc.p_env, fy, fx;
        const uint32_t y = alias_pick(sc.env_rows, bin_of(u1, sc.eh, fy), d);
        const uint32_t x = alias_pick(sc.env_cols + (size_t)y * sc.ew, bin_of(u2, sc.ew, fx), d);
#else
        uint32_t y = upper_bound_f(sc.env_marg + 1, sc.eh, u1, sc.env_marg_guide, sc.env_marg_g);
        y = min(y, sc.eh - 1u);
        const float m0 = __ldg(&sc.env_marg[y]), m1 = __ldg(&sc.env_marg[y + 1]);
        const float* c = sc.env_cond + (size_t)y * (sc.ew + 1);
        uint32_t x = upper_bound_f(c + 1, sc.ew, u2,
                                   sc.env_cond_guide + (size_t)y * (sc.env_cond_g + 1u),
                                   sc.env_cond_g);
        x = min(x, sc.ew - 1u);
        const float c0 = __ldg(&c[x]), c1 = __ldg(&c[x + 1]);
        const float fy = fminf(fmaxf((u1 - m0) / (m1 - m0), 0.f), 1.f);
        const float fx = fminf(fmaxf((u2 - c0) / (c1 - c0), 0.f), 1.f);
#endif
        const float u = ((float)x + fx) / (float)sc.ew, v = ((float)y + fy) / (float)sc.eh;
        // phi = pi (2u - 1), theta = pi v: sine and cosine of pi times an argument in [-1, 1]
        float sp, cp, st, ct;
        sincospif(2.0f * u - 1.0f, &sp, &cp);
        sincospif(v, &st, &ct);
        const float3 dl = f3(st * sp, ct, -st * cp);
        const float* M = sc.env_m;
        const float3 dw = f3(M[0] * dl.x + M[3] * dl.y + M[6] * dl.z,
                             M[1] * dl.x + M[4] * dl.y + M[7] * dl.z,
                             M[2] * dl.x + M[5] * dl.y + M[8] * dl.z);
        ls.dir = normalize(dw);
        ls.dist = kRayTmax;
        // radiance and density at the sampled map point itself (the direction maps back to it
        // up to rounding), without the inverse trigonometry of a lookup by direction
        ls.le = env_eval_uv(sc, u, v);
        ls.pdf = sc.p_env * env_pdf_st(sc, u, v, st);
        ls.valid = ls.pdf > 0.f;
        return ls;
    }
    const float ut = sc.p_env > 0.f ? (u0 - sc.p_env) / (1.0f - sc.p_env) : u0;
    uint32_t k = upper_bound_f(sc.light_cdf, sc.n_lights, ut, sc.light_guide, sc.light_g);
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

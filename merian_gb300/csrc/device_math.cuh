// Device arithmetic of the `pt` path: vectors, RNG, encodings, frames, camera, Fresnel, GGX and
// the material BSDFs, as sm_103a device functions. Each function names the merian source it
// computes the same quantity as (paths relative to the merian project root).
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace gbpt {

#define GBPT_DI __device__ __forceinline__

// ---- float3 -----------------------------------------------------------------------------------
GBPT_DI float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
GBPT_DI float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
GBPT_DI float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
GBPT_DI float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
GBPT_DI float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
GBPT_DI float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
GBPT_DI float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
GBPT_DI float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
GBPT_DI float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GBPT_DI float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
GBPT_DI float length(float3 a) { return sqrtf(dot(a, a)); }
GBPT_DI float3 normalize(float3 a) {
    const float l = sqrtf(dot(a, a));
    return f3(a.x / l, a.y / l, a.z / l);
}
GBPT_DI float lerpf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
GBPT_DI float3 lerp3(float3 x, float3 y, float a) {
    return f3(lerpf(x.x, y.x, a), lerpf(x.y, y.y, a), lerpf(x.z, y.z, a));
}
GBPT_DI float pow2(float x) { return x * x; }
GBPT_DI float signf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
GBPT_DI float max3(float3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
GBPT_DI bool all_zero(float3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 6.28318530717958647692f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kInv2Pi = 0.15915494309189533577f;
constexpr float kBsdfMinCos = 1e-6f;        // bsdf.slang:13
constexpr float kThroughputMin = 1e-5f;     // scene.slang:24
constexpr float kRayTmax = 1e7f;            // hit.slang:8
constexpr float kEnvDistance = 1e7f;        // environment-map.slang:12
constexpr float kMinAlpha = 0.0316f * 0.0316f; // material.slang:23 (roughness^2)
// pdf of a delta lobe; a mix passes such a sample through (w f1 / (w p1) = its own weight)
constexpr float kInf = __builtin_huge_valf();

// ---- RNG --------------------------------------------------------------------------------------
// pcg4d16 (utils/hash.slang:138-147)
GBPT_DI uint32_t pcg4d16(uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
    x = x * 1664525u + 1013904223u;
    y = y * 1664525u + 1013904223u;
    z = z * 1664525u + 1013904223u;
    w = w * 1664525u + 1013904223u;
    x += y * w;
    y += z * x;
    z += x * y;
    w += y * z;
    x += y * w;
    return x;
}
// PCG::next (utils/random.slang:108-128) and uint_to_zero_one_float_rust (bit-twiddling.slang:23)
struct Pcg {
    uint32_t state;
    GBPT_DI uint32_t next() {
        const uint32_t s = state;
        state = state * 747796405u + 2891336453u;
        const uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
        return (word >> 22u) ^ word;
    }
    GBPT_DI float next_float() { return (float)(next() >> 8) * 5.9604644775390625e-08f; }
};
// XorShift32 (utils/random.slang:64-80), used by the BSDF property checks
struct XorShift {
    uint32_t state;
    GBPT_DI uint32_t next() {
        uint32_t v = state;
        v ^= v << 13u;
        v ^= v >> 17u;
        v ^= v << 5u;
        state = v;
        return v;
    }
    GBPT_DI float next_float() { return (float)(next() >> 8) * 5.9604644775390625e-08f; }
};

// ---- encodings (utils/encoding.slang:6-55) ------------------------------------------------------
GBPT_DI float unpack_snorm16(uint32_t b) {
    const float f = (float)(int16_t)(uint16_t)b / 32767.0f;
    return fminf(fmaxf(f, -1.0f), 1.0f);
}
GBPT_DI float3 decode_normal(uint32_t enc) {
    float x = unpack_snorm16(enc & 0xffffu), y = unpack_snorm16(enc >> 16);
    const float z = (1.0f - fabsf(x)) - fabsf(y);
    if (z < 0.0f) {
        const float nx = copysignf(1.0f - fabsf(y), x);
        const float ny = copysignf(1.0f - fabsf(x), y);
        x = nx;
        y = ny;
    }
    return normalize(f3(x, y, z));
}
GBPT_DI uint32_t pack_snorm16(float v) {
    v = fminf(fmaxf(v, -1.0f), 1.0f);
    return (uint32_t)(uint16_t)(int16_t)__float2int_rn(roundf(v * 32767.0f));
}
GBPT_DI uint32_t encode_normal(float3 n) {
    const float inv = 1.0f / ((fabsf(n.x) + fabsf(n.y)) + fabsf(n.z));
    float px, py;
    if (n.z < 0.0f) {
        px = copysignf(1.0f - fabsf(n.y * inv), n.x);
        py = copysignf(1.0f - fabsf(n.x * inv), n.y);
    } else {
        px = n.x * inv;
        py = n.y * inv;
    }
    return pack_snorm16(px) | (pack_snorm16(py) << 16);
}
GBPT_DI float half_lo(uint32_t h2) { return __half2float(__ushort_as_half((unsigned short)(h2 & 0xffffu))); }
GBPT_DI float half_hi(uint32_t h2) { return __half2float(__ushort_as_half((unsigned short)(h2 >> 16))); }
GBPT_DI float round_half(float x) { return __half2float(__float2half_rn(x)); }

// ---- frames (utils/frame.slang) ------------------------------------------------------------------
struct Frame {
    float3 t, b, n;
    GBPT_DI float3 to_local(float3 v) const { return f3(dot(t, v), dot(b, v), dot(n, v)); }
    GBPT_DI float3 to_world(float3 v) const {
        return f3(v.x * t.x + v.y * b.x + v.z * n.x, v.x * t.y + v.y * b.y + v.z * n.y,
                  v.x * t.z + v.y * b.z + v.z * n.z);
    }
};
// make_frame, Duff et al. 2017 (frame.slang:7-13)
GBPT_DI Frame frame_from_normal(float3 z) {
    const float sgn = (z.z >= 0.f) ? 1.f : -1.f;
    const float a = -1.0f / (sgn + z.z);
    const float b = z.x * z.y * a;
    Frame f;
    f.t = f3(1.0f + sgn * z.x * z.x * a, sgn * b, -sgn * z.x);
    f.b = f3(b, sgn + z.y * z.y * a, -z.y);
    f.n = z;
    return f;
}
// OrthonormalFrame(n, tangent, handedness) (frame.slang:90-95)
GBPT_DI Frame frame_from_tangent(float3 n, float3 tg, float hand) {
    const float3 N = normalize(n);
    const float3 T = normalize(tg - N * dot(tg, N));
    Frame f;
    f.t = T;
    f.b = cross(N, T) * hand;
    f.n = N;
    return f;
}
// apply_normal_map(float3(0,0,1)) (frame.slang:126-134): re-orthonormalised, right-handed
GBPT_DI Frame reorthonormalize(const Frame& f) {
    const float3 nN = f.to_world(f3(0.f, 0.f, 1.f));
    const float3 nT = normalize(f.t - nN * dot(f.t, nN));
    Frame r;
    r.t = nT;
    r.b = cross(nN, nT);
    r.n = nN;
    return r;
}

// ---- ray offset (hit.slang:14-23, Waechter & Binder) ----------------------------------------------
GBPT_DI float offset_axis(float p, float n) {
    const int io = (int)(n * 256.0f);
    const float ip = __int_as_float(__float_as_int(p) + (p < 0.0f ? -io : io));
    return fabsf(p) < (1.0f / 16.0f) ? p + n * (1.0f / 65536.0f) : ip;
}
GBPT_DI float3 offset_ray_origin(float3 p, float3 n) {
    return f3(offset_axis(p.x, n.x), offset_axis(p.y, n.y), offset_axis(p.z, n.z));
}

// ---- Fresnel (utils/fresnel.slang:14-42) ----------------------------------------------------------
GBPT_DI float schlick_term(float c) { return powf(fmaxf(1.0f - c, 0.0f), 5.0f); }
GBPT_DI float fresnel_dielectric(float cos_i, float eta) {
    const float sin2_t = eta * eta * (1.0f - cos_i * cos_i);
    if (sin2_t >= 1.0f) return 1.0f;
    const float cos_t = sqrtf(1.0f - sin2_t);
    const float r_parl = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const float r_perp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return 0.5f * (r_parl * r_parl + r_perp * r_perp);
}
GBPT_DI float3 reflect2(float3 i, float3 n, float ndoti) { return (2.0f * ndoti) * n - i; }
GBPT_DI float3 refract3(float3 i, float3 n, float eta) { // HLSL refract
    const float ni = dot(n, i);
    const float k = 1.0f - eta * eta * (1.0f - ni * ni);
    if (k < 0.0f) return f3(0.f, 0.f, 0.f);
    return eta * i - (eta * ni + sqrtf(k)) * n;
}

// ---- GGX (shading/bsdfs/brdf-ggx.slang) -----------------------------------------------------------
GBPT_DI float g1_over_s(float widotn, float a2) {
    return 2.0f / (widotn + sqrtf(a2 + ((1.0f - a2) * (widotn * widotn))));
}
GBPT_DI float g2_over_s(float wodotn, float widotn, float a2) {
    const float g1 = widotn * sqrtf(a2 + ((1.0f - a2) * (wodotn * wodotn)));
    const float g2 = wodotn * sqrtf(a2 + ((1.0f - a2) * (widotn * widotn)));
    return (2.0f * wodotn) / (g1 + g2);
}
GBPT_DI float g1_over_v(float3 wi, float ax, float ay) {
    return 2.0f / (wi.z + length(f3(ax * wi.x, ay * wi.y, wi.z)));
}
GBPT_DI float g2_over_v(float3 wo, float3 wi, float ax, float ay) {
    const float g1 = wi.z * length(f3(ax * wo.x, ay * wo.y, wo.z));
    const float g2 = wo.z * length(f3(ax * wi.x, ay * wi.y, wi.z));
    return (2.0f * wo.z) / (g1 + g2);
}
GBPT_DI float ndf_s(float ndoth2, float a2) {
    return a2 / (kPi * pow2((ndoth2 * a2) + (1.0f - ndoth2)));
}
GBPT_DI float ndf_v(float3 h, float ax, float ay) {
    const float axy = ax * ay;
    const float3 v = f3(ay * h.x, ax * h.y, axy * h.z);
    const float w2 = axy / dot(v, v);
    return axy * w2 * w2 / kPi;
}
// Dupuy & Benyoub 2023 spherical-cap VNDF sampling (brdf-ggx.slang:137-152)
GBPT_DI float3 vndf_sample(float3 wi, float ax, float ay, float r0, float r1) {
    const float3 ws = normalize(f3(wi.x * ax, wi.y * ay, wi.z));
    const float phi = ((2.0f * r0) - 1.0f) * kPi;
    const float z = fmaf(1.0f - r1, 1.0f + ws.z, -ws.z);
    const float st = sqrtf(fminf(fmaxf(1.0f - (z * z), 0.0f), 1.0f));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float3 m = f3(st * cp, st * sp, z) + ws;
    return normalize(f3(m.x * ax, m.y * ay, m.z));
}
GBPT_DI float vndf_pdf_wo_v(float3 wi, float3 h, float ax, float ay) {
    return (ndf_v(h, ax, ay) * g1_over_v(wi, ax, ay)) / 4.0f;
}
GBPT_DI float vndf_pdf_wo_s(float widotn, float ndoth2, float a2) {
    return (ndf_s(ndoth2, a2) * g1_over_s(widotn, a2)) / 4.0f;
}
GBPT_DI float vndf_h_pdf(float3 wi, float3 h, float a2) {
    return ndf_s(h.z * h.z, a2) * g1_over_s(wi.z, a2) * fmaxf(0.0f, dot(wi, h));
}

struct BsdfSample {
    float3 wo;
    float pdf;
    float3 weight;
    bool valid;
};
GBPT_DI BsdfSample no_sample() {
    BsdfSample s;
    s.valid = false;
    s.wo = f3(0.f, 0.f, 0.f);
    s.pdf = 0.f;
    s.weight = f3(0.f, 0.f, 0.f);
    return s;
}
GBPT_DI BsdfSample mk_sample(float3 wo, float pdf, float3 w) {
    BsdfSample s;
    s.wo = wo;
    s.pdf = pdf;
    s.weight = w;
    s.valid = true;
    return s;
}

// LambertDiffuseBRDF (brdf-lambert-diffuse.slang:32-90), sample_cos (utils/sampling.slang:24-29)
template <class G> GBPT_DI BsdfSample lambert_sample(float3 albedo, float3 wi, G& rng) {
    const float x0 = rng.next_float(), x1 = rng.next_float();
    const float su = sqrtf(x0);
    float sp, cp;
    sincosf(kTwoPi * x1, &sp, &cp);
    const float3 wo = f3(su * cp, su * sp, sqrtf(1.0f - x0));
    if (fminf(wi.z, wo.z) < kBsdfMinCos) return no_sample();
    return mk_sample(wo, kInvPi * wo.z, albedo);
}
GBPT_DI float3 lambert_eval(float3 albedo, float3 wi, float3 wo) {
    if (fminf(wi.z, wo.z) < kBsdfMinCos) return f3(0.f, 0.f, 0.f);
    return (kInvPi * albedo) * wo.z;
}
GBPT_DI float lambert_pdf(float3 wi, float3 wo) {
    if (fminf(wi.z, wo.z) < kBsdfMinCos) return 0.0f;
    return kInvPi * wo.z;
}

// GGXBRDF (brdf-ggx.slang:331-397)
template <class G> GBPT_DI BsdfSample ggx_sample(float ax, float ay, float3 wi, G& rng) {
    if (wi.z < kBsdfMinCos) return no_sample();
    const float r0 = rng.next_float(), r1 = rng.next_float();
    const float3 h = vndf_sample(wi, ax, ay, r0, r1);
    const float3 wo = reflect2(wi, h, dot(wi, h));
    if (wo.z < kBsdfMinCos) return no_sample();
    const float pdf = vndf_pdf_wo_v(wi, h, ax, ay);
    const float w = g2_over_v(wo, wi, ax, ay) / g1_over_v(wi, ax, ay);
    return mk_sample(wo, pdf, f3(w, w, w));
}
GBPT_DI float ggx_eval(float ax, float ay, float3 wi, float3 wo) {
    if (fminf(wi.z, wo.z) < kBsdfMinCos) return 0.0f;
    const float3 h = normalize(wo + wi);
    return (ndf_v(h, ax, ay) * g2_over_v(wo, wi, ax, ay)) / 4.0f;
}
GBPT_DI float ggx_pdf(float ax, float ay, float3 wi, float3 wo) {
    if (fminf(wi.z, wo.z) < kBsdfMinCos) return 0.0f;
    const float3 h = normalize(wi + wo);
    return vndf_pdf_wo_v(wi, h, ax, ay);
}

// ConductorFresnelBSDF<GGXBRDF> (bsdf-conductor-fresnel.slang:6-37)
GBPT_DI float3 schlick3(float3 f0, float c) {
    const float t = schlick_term(c);
    return f0 + (f3(1.f, 1.f, 1.f) - f0) * t;
}
template <class G>
GBPT_DI BsdfSample conductor_sample(float ax, float ay, float3 f0, float3 wi, G& rng) {
    BsdfSample s = ggx_sample(ax, ay, wi, rng);
    if (!s.valid) return s;
    const float3 h = normalize(wi + s.wo);
    s.weight = s.weight * schlick3(f0, dot(wi, h));
    return s;
}
GBPT_DI float3 conductor_eval(float ax, float ay, float3 f0, float3 wi, float3 wo) {
    const float3 h = normalize(wi + wo);
    return schlick3(f0, dot(wi, h)) * ggx_eval(ax, ay, wi, wo);
}

// Index-matched boundary: |eta - 1| < 1e-3 (the IOR bookkeeping yields 0.99999994 as often as 1).
// Its transmission is a delta lobe: sampling reports pdf = inf, evaluation sees no lobe.
GBPT_DI bool index_matched(float eta) { return fabsf(eta - 1.0f) < 1e-3f; }

// RoughDielectricBSDF (bsdf-rough-dielectric.slang:65-161)
template <class G>
GBPT_DI BsdfSample rough_dielectric_sample(float alpha, float eta, float3 tint, float3 wi, G& rng) {
    if (wi.z < kBsdfMinCos) return no_sample();
    const float a2 = pow2(alpha);
    const float r0 = rng.next_float(), r1 = rng.next_float();
    const float3 wm = vndf_sample(wi, alpha, alpha, r0, r1);
    const float widoth = dot(wi, wm);
    const float R = fresnel_dielectric(fabsf(widoth), eta);
    if (rng.next_float() < R) {
        const float3 wo = reflect2(wi, wm, widoth);
        if (wo.z < kBsdfMinCos) return no_sample();
        const float w = g2_over_s(wo.z, wi.z, a2) / g1_over_s(wi.z, a2);
        const float pdf = R * vndf_pdf_wo_s(wi.z, pow2(wm.z), a2);
        return mk_sample(wo, pdf, f3(w, w, w));
    }
    const float3 wo = refract3(-wi, wm, eta);
    if (all_zero(wo) || wo.z > -kBsdfMinCos) return no_sample();
    const float wodoth = dot(wo, wm);
    const float denom = wodoth + eta * widoth;
    const float pdf = index_matched(eta)
                          ? __int_as_float(0x7f800000)
                          : (1.0f - R) * vndf_h_pdf(wi, wm, a2) * fabsf(wodoth) / pow2(denom);
    const float w = pow2(eta) * g2_over_s(fabsf(wo.z), wi.z, a2) / g1_over_s(wi.z, a2);
    return mk_sample(wo, pdf, tint * w);
}
GBPT_DI float3 rough_dielectric_eval(float alpha, float eta, float3 tint, float3 wi, float3 wo) {
    if (wi.z < kBsdfMinCos) return f3(0.f, 0.f, 0.f);
    if (wo.z > kBsdfMinCos) {
        const float3 h = normalize(wi + wo);
        const float R = fresnel_dielectric(fabsf(dot(wi, h)), eta);
        const float g = R * ggx_eval(alpha, alpha, wi, wo);
        return f3(g, g, g);
    }
    // index-matched boundary: the transmission is a delta only sampling produces, so evaluation
    // (next-event estimation, MIS) sees no transmission lobe
    if (wo.z < -kBsdfMinCos && !index_matched(eta)) {
        float3 h = normalize(wo + wi * eta);
        h = h * signf(h.z);
        // only a microfacet seen from its front by wi and left through its back by wo refracts
        // wi into wo; the other configurations are never sampled, so they carry no density here
        if (!(dot(wi, h) > 0.0f && dot(wo, h) < 0.0f)) return f3(0.f, 0.f, 0.f);
        const float R = fresnel_dielectric(fabsf(dot(wi, h)), eta);
        // GGXBTDF::eval (brdf-ggx.slang:427-444)
        const float widoth = dot(wi, h), wodoth = dot(wo, h);
        const float a2 = pow2(alpha);
        const float g2 = g2_over_s(fabsf(wo.z), wi.z, a2);
        const float d = ndf_s(pow2(h.z), a2);
        const float denom = wodoth + (eta * widoth);
        const float jac = pow2(eta) * widoth * wodoth / pow2(denom);
        return (1.0f - R) * (tint * (d * g2 * fabsf(jac)));
    }
    return f3(0.f, 0.f, 0.f);
}
GBPT_DI float rough_dielectric_pdf(float alpha, float eta, float3 wi, float3 wo) {
    if (wi.z < kBsdfMinCos) return 0.0f;
    const float a2 = pow2(alpha);
    if (wo.z > kBsdfMinCos) {
        const float3 h = normalize(wi + wo);
        const float R = fresnel_dielectric(fabsf(dot(wi, h)), eta);
        return R * vndf_pdf_wo_s(wi.z, pow2(fmaxf(0.0f, h.z)), a2);
    }
    if (wo.z < -kBsdfMinCos && !index_matched(eta)) { // else a delta transmission
        float3 h = normalize(wo + wi * eta);
        h = h * signf(h.z);
        if (!(dot(wi, h) > 0.0f && dot(wo, h) < 0.0f)) return 0.0f; // as the eval
        const float R = fresnel_dielectric(fabsf(dot(wi, h)), eta);
        const float wodoth = dot(wo, h);
        const float denom = wodoth + eta * dot(wi, h);
        return (1.0f - R) * vndf_h_pdf(wi, h, a2) * fabsf(wodoth) / pow2(denom);
    }
    return 0.0f;
}

// ---- material instance at a shading point ---------------------------------------------------------
// DiffuseMaterial (diffuse-material.slang:7-43) or the OpenPBR substrate
// MixBSDF<MixBSDF<FresnelMixBSDF<GGX, Lambert>, RoughDielectric>, ConductorFresnel<GGX>>
// (openpbr-material.slang:133-136,220-323). Clear coat and sheen are compile-time absent for these
// models, so their weight-0 mixes are the identity. A runtime mix weight of exactly 0 or 1 skips
// the other lobe's evaluation: lerp(x, y, 0) = x and lerp(x, y, 1) = y for finite x, y.
struct Material {
    uint32_t model; // GBPT_MATERIAL_*
    float3 base;
    float ax, ay;
    float f0;       // dielectric specular F0
    float metal;    // substrate mix weight
    float tw;       // transmission mix weight
    float eta;      // interior relative IOR
    float alpha_iso;
    float3 tcol;
};

GBPT_DI float opaque_F(float f0, float c) { return f0 + (1.0f - f0) * schlick_term(c); }
// FresnelMixBSDF<GGX, Lambert> (bsdf-fresnel-mix.slang:7-63)
GBPT_DI float3 opaque_eval(const Material& m, float3 wi, float3 wo) {
    const float3 h = normalize(wi + wo);
    const float F = opaque_F(m.f0, dot(wi, h));
    const float g = ggx_eval(m.ax, m.ay, wi, wo);
    return lerp3(lambert_eval(m.base, wi, wo), f3(g, g, g), F);
}
GBPT_DI float opaque_pdf(const Material& m, float3 wi, float3 wo) {
    const float F = opaque_F(m.f0, wi.z);
    return lerpf(lambert_pdf(wi, wo), ggx_pdf(m.ax, m.ay, wi, wo), F);
}
template <class G> GBPT_DI BsdfSample opaque_sample(const Material& m, float3 wi, G& rng) {
    const float F = opaque_F(m.f0, wi.z);
    const BsdfSample s = rng.next_float() < F ? ggx_sample(m.ax, m.ay, wi, rng)
                                              : lambert_sample(m.base, wi, rng);
    if (!s.valid) return s;
    const float p = opaque_pdf(m, wi, s.wo);
    return mk_sample(s.wo, p, opaque_eval(m, wi, s.wo) / p);
}

// Power-heuristic weight of density a against density b as 1 / (1 + (b/a)^2): an unbounded a (a
// near-delta lobe) gives 1 instead of inf/inf.
GBPT_DI float power_heuristic(float a, float b) {
    if (!(a > 0.0f)) return 0.0f;
    const float r = b / a;
    return 1.0f / (1.0f + r * r);
}

// MixBSDF<OpaqueDielectric, RoughDielectric>(tw). A mix weight of exactly 0 or 1 passes the
// sampled lobe through: lerp(x, y, 1) = y and (weight * pdf) / pdf = weight, evaluated exactly
// (rounded, the round trip turns the unbounded pdf of an index-matched refraction into NaN).
GBPT_DI float3 dielectric_eval(const Material& m, float3 wi, float3 wo) {
    if (m.tw == 0.0f) return opaque_eval(m, wi, wo);
    if (m.tw == 1.0f) return rough_dielectric_eval(m.alpha_iso, m.eta, m.tcol, wi, wo);
    return lerp3(opaque_eval(m, wi, wo), rough_dielectric_eval(m.alpha_iso, m.eta, m.tcol, wi, wo),
                 m.tw);
}
GBPT_DI float dielectric_pdf(const Material& m, float3 wi, float3 wo) {
    if (m.tw == 0.0f) return opaque_pdf(m, wi, wo);
    if (m.tw == 1.0f) return rough_dielectric_pdf(m.alpha_iso, m.eta, wi, wo);
    return lerpf(opaque_pdf(m, wi, wo), rough_dielectric_pdf(m.alpha_iso, m.eta, wi, wo), m.tw);
}
template <class G> GBPT_DI BsdfSample dielectric_sample(const Material& m, float3 wi, G& rng) {
    if (m.tw > 0.0f && rng.next_float() < m.tw) {
        const BsdfSample s = rough_dielectric_sample(m.alpha_iso, m.eta, m.tcol, wi, rng);
        if (!s.valid || m.tw == 1.0f || !(s.pdf < kInf)) return s;
        const float mp = lerpf(opaque_pdf(m, wi, s.wo), s.pdf, m.tw);
        const float3 me = lerp3(opaque_eval(m, wi, s.wo), s.weight * s.pdf, m.tw);
        return mk_sample(s.wo, mp, me / mp);
    }
    const BsdfSample s = opaque_sample(m, wi, rng);
    if (!s.valid || m.tw == 0.0f || !(s.pdf < kInf)) return s;
    const float mp = lerpf(s.pdf, rough_dielectric_pdf(m.alpha_iso, m.eta, wi, s.wo), m.tw);
    const float3 me =
        lerp3(s.weight * s.pdf, rough_dielectric_eval(m.alpha_iso, m.eta, m.tcol, wi, s.wo), m.tw);
    return mk_sample(s.wo, mp, me / mp);
}

GBPT_DI float3 material_eval(const Material& m, float3 wi, float3 wo) {
    if (m.model == 0u) return lambert_eval(m.base, wi, wo);
    if (m.metal == 1.0f) return conductor_eval(m.ax, m.ay, m.base, wi, wo);
    if (m.metal == 0.0f) return dielectric_eval(m, wi, wo);
    return lerp3(dielectric_eval(m, wi, wo), conductor_eval(m.ax, m.ay, m.base, wi, wo), m.metal);
}
GBPT_DI float material_pdf(const Material& m, float3 wi, float3 wo) {
    if (m.model == 0u) return lambert_pdf(wi, wo);
    if (m.metal == 1.0f) return ggx_pdf(m.ax, m.ay, wi, wo);
    if (m.metal == 0.0f) return dielectric_pdf(m, wi, wo);
    return lerpf(dielectric_pdf(m, wi, wo), ggx_pdf(m.ax, m.ay, wi, wo), m.metal);
}
template <class G> GBPT_DI BsdfSample material_sample(const Material& m, float3 wi, G& rng) {
    if (m.model == 0u) return lambert_sample(m.base, wi, rng);
    if (m.metal > 0.0f && rng.next_float() < m.metal) {
        const BsdfSample s = conductor_sample(m.ax, m.ay, m.base, wi, rng);
        if (!s.valid || m.metal == 1.0f || !(s.pdf < kInf)) return s;
        const float mp = lerpf(dielectric_pdf(m, wi, s.wo), s.pdf, m.metal);
        const float3 me = lerp3(dielectric_eval(m, wi, s.wo), s.weight * s.pdf, m.metal);
        return mk_sample(s.wo, mp, me / mp);
    }
    const BsdfSample s = dielectric_sample(m, wi, rng);
    if (!s.valid || m.metal == 0.0f || !(s.pdf < kInf)) return s;
    const float mp = lerpf(s.pdf, ggx_pdf(m.ax, m.ay, wi, s.wo), m.metal);
    const float3 me = lerp3(s.weight * s.pdf, conductor_eval(m.ax, m.ay, m.base, wi, s.wo), m.metal);
    return mk_sample(s.wo, mp, me / mp);
}

GBPT_DI float yuv_luminance(float3 c) { return dot(c, f3(0.299f, 0.587f, 0.114f)); }

// Directional albedo fit of GGX with height-correlated Smith G2 (ggx_integral_approx_ and
// ggx_integral_approx_correlated, brdf-ggx.slang:285-316): bias and scale are ratios of
// polynomials in (cos theta, alpha), the bias suppressed for F0 near 0. The coefficient rows are
// the reference's fit (row-major, mul(M, x) = rows . x).
GBPT_DI float3 ggx_preintegrated(float3 F0, float alpha, float cos_theta) {
    const float c = fabsf(cos_theta), c2 = c * c, c3 = c2 * c;
    const float a = alpha, a2 = a * a, a3 = a2 * a;
    const float n1 = (0.995367f + -1.38839f * c) + (-0.24751f + 1.97442f * c) * a;
    const float d1 = (1.0f + 2.68132f * c + 52.366f * c3) +
                     (16.0932f + -3.98452f * c + 59.3013f * c3) * a +
                     (-5.18731f + 255.259f * c + 2544.07f * c3) * a3;
    const float n2 = (-0.0564526f + 3.82901f * c) + (16.91f + -11.0303f * c) * a;
    const float d2 = (1.0f + 4.11118f * c2 + -1.37886f * c3) +
                     (19.3254f + -28.9947f * c2 + 16.9514f * c3) * a +
                     (0.545386f + 96.0994f * c2 + -79.4492f * c3) * a3;
    float bias = n1 / d1;
    const float scale = n2 / d2;
    const float luma = (F0.x + F0.y + F0.z) * (1.0f / 3.0f);
    bias *= fminf(fmaxf(luma * 50.0f, 0.0f), 1.0f);
    const float sc = fmaxf(0.0f, scale), b = fmaxf(0.0f, bias);
    return f3(F0.x * sc + b, F0.y * sc + b, F0.z * sc + b);
}

// BSDF::get_albedo of the material toward wi (the GBuffer's albedo): Lambert albedo
// (brdf-lambert-diffuse.slang:50-52); conductor, Fresnel mix, rough dielectric and mix as
// bsdf-conductor-fresnel.slang:39-41, bsdf-fresnel-mix.slang:50-53,
// bsdf-rough-dielectric.slang:111-115, bsdf-mix.slang:51-54.
GBPT_DI float3 material_albedo(const Material& m, float3 wi) {
    if (m.model == 0u) return m.base;
    const float a_xy = sqrtf(m.ax * m.ay);
    const float3 one = f3(1.f, 1.f, 1.f);
    const float3 spec = ggx_preintegrated(f3(m.f0, m.f0, m.f0), a_xy, wi.z);
    const float3 opaque = spec + (one - spec) * m.base;
    const float fd = ((1.0f - m.eta) / (1.0f + m.eta)) * ((1.0f - m.eta) / (1.0f + m.eta));
    const float3 sd = ggx_preintegrated(f3(fd, fd, fd), sqrtf(m.alpha_iso * m.alpha_iso), wi.z);
    const float3 diel = sd + (one - sd) * (m.eta * m.eta * m.tcol);
    const float3 cond = ggx_preintegrated(m.base, a_xy, wi.z);
    return lerp3(lerp3(opaque, diel, m.tw), cond, m.metal);
}

// OpenPBRMaterial::get_sample / DiffuseMaterial::get_sample (openpbr-material.slang:220-323,
// diffuse-material.slang:27-41) from the first four float4 of a gbpt_material record: model and
// base colour, (metalness, alpha_x, alpha_y, specular_weight), (specular_ior, emission),
// (transmission_weight, transmission_color). `ior` is the path's current IOR.
GBPT_DI Material material_from_record(float4 m0, float4 m1, float4 m2, float4 m3, bool front,
                                      float ior) {
    Material m;
    m.model = __float_as_uint(m0.x);
    m.base = f3(m0.y, m0.z, m0.w);
    m.eta = 1.0f;
    m.tw = 0.f;
    m.tcol = f3(1.f, 1.f, 1.f);
    if (m.model == 0u) {
        m.ax = m.ay = 1.f;
        m.f0 = 0.f;
        m.metal = 0.f;
        m.alpha_iso = 1.f;
        return m;
    }
    m.metal = m1.x;
    m.ax = fmaxf(m1.y, kMinAlpha);
    m.ay = fmaxf(m1.z, kMinAlpha);
    const float sior = m2.x;
    const float ior_t = (sior - 1.0f) / (sior + 1.0f);
    m.f0 = fminf(fmaxf(m1.w * ior_t * ior_t, 0.0f), 1.0f);
    const bool transmission = m.model == 2u;
    if (transmission) {
        m.eta = ior / (front ? sior : 1.0f);
        m.tw = m3.x;
        m.tcol = f3(m3.y, m3.z, m3.w);
    }
    m.alpha_iso = transmission ? sqrtf(m.ax * m.ay) : m.ax;
    return m;
}

} // namespace gbpt

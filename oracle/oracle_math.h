// ORACLE (test infrastructure only). CPU restatement of the arithmetic of merian's `pt` path:
// vector helpers, RNG, encodings, camera, BSDFs and materials. Templated on the real type R so
// the same source builds the FP64 parity estimator and the FP32 CPU baseline. Each function
// cites the reference file:line it restates (paths relative to the merian project root).
// Compiled with -ffp-contract=off so FP32 results do not depend on the host's FMA contraction.
#pragma once

#include "gbpt.h"

#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

template <class R> struct V3 {
    R x, y, z;
};
template <class R> inline V3<R> mk(R x, R y, R z) { return {x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
// normalize(v) = v / |v|
template <class R> inline V3<R> normalize(V3<R> a) {
    const R l = std::sqrt(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}
// HLSL/GLSL mix semantics x*(1-a) + y*a
template <class R> inline R lerp(R x, R y, R a) { return x * (R(1) - a) + y * a; }
template <class R> inline V3<R> lerp(V3<R> x, V3<R> y, R a) {
    return {lerp(x.x, y.x, a), lerp(x.y, y.y, a), lerp(x.z, y.z, a)};
}
template <class R> inline R pow2(R x) { return x * x; }
template <class R> inline R clampr(R x, R lo, R hi) { return x < lo ? lo : (x > hi ? hi : x); }
template <class R> inline R maxr(R a, R b) { return a > b ? a : b; }
template <class R> inline R minr(R a, R b) { return a < b ? a : b; }
template <class R> inline R signr(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }

template <class R> struct C {
    static constexpr R PI = R(3.14159265358979323846);
    static constexpr R TWO_PI = R(6.28318530717958647692);
    static constexpr R INV_PI = R(0.31830988618379067154);
    static constexpr R INV_2PI = R(0.15915494309189533577);
};

inline float as_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline uint32_t as_uint(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// ---- RNG ---------------------------------------------------------------------------------------
// pcg4d16 (include/merian-shaders/utils/hash.slang:138-147)
inline uint32_t pcg4d16(uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
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
// uint_to_zero_one_float_rust (utils/bit-twiddling.slang:23-27)
inline float u01(uint32_t u) { return (float)(u >> 8) * 5.9604644775390625e-08f; }

// PCG::next (utils/random.slang:108-128)
struct Pcg {
    uint32_t state;
    uint32_t next() {
        const uint32_t s = state;
        state = state * 747796405u + 2891336453u;
        const uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
        return (word >> 22u) ^ word;
    }
    float next_float() { return u01(next()); }
};
// XorShift32 (utils/random.slang:64-80, hash.slang:190-196), used by the BSDF checks
struct XorShift {
    uint32_t state;
    uint32_t next() {
        uint32_t v = state;
        v ^= v << 13u;
        v ^= v >> 17u;
        v ^= v << 5u;
        state = v;
        return v;
    }
    float next_float() { return u01(next()); }
};

// ---- encodings (utils/encoding.slang:6-55) ------------------------------------------------------
inline float unpack_snorm16(uint32_t bits16) {
    const int16_t i = (int16_t)(uint16_t)bits16;
    float f = (float)i / 32767.0f;
    return f < -1.0f ? -1.0f : (f > 1.0f ? 1.0f : f);
}
inline uint32_t pack_snorm16(float v) {
    v = v < -1.0f ? -1.0f : (v > 1.0f ? 1.0f : v);
    return (uint32_t)(uint16_t)(int16_t)(int32_t)std::round(v * 32767.0f);
}
// decode_normal: float decode then normalize, in R
template <class R> inline V3<R> decode_normal(uint32_t enc) {
    const float px = unpack_snorm16(enc & 0xffffu), py = unpack_snorm16(enc >> 16);
    R x = (R)px, y = (R)py;
    R z = (R(1) - std::fabs(x)) - std::fabs(y);
    if (z < R(0)) {
        const R nx = std::copysign(R(1) - std::fabs(y), x);
        const R ny = std::copysign(R(1) - std::fabs(x), y);
        x = nx;
        y = ny;
    }
    return normalize(mk(x, y, z));
}
// encode_normal: octahedral_project + packSnorm2x16 (computed in float, as the reference stores
// the encoding as a 32-bit word)
inline uint32_t encode_normal(float nx, float ny, float nz) {
    const float inv = 1.0f / ((std::fabs(nx) + std::fabs(ny)) + std::fabs(nz));
    float px, py;
    if (nz < 0.0f) {
        px = std::copysign(1.0f - std::fabs(ny * inv), nx);
        py = std::copysign(1.0f - std::fabs(nx * inv), ny);
    } else {
        px = nx * inv;
        py = ny * inv;
    }
    return pack_snorm16(px) | (pack_snorm16(py) << 16);
}

inline float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    if (e == 0) {
        const float v = (float)m * 5.9604644775390625e-08f; // 2^-24
        return sign ? -v : v;
    }
    if (e == 31) return as_float(sign | 0x7f800000u | (m << 13));
    return as_float(sign | ((e + 112u) << 23) | (m << 13));
}
// round to nearest even, as Slang's float -> half conversion
inline uint16_t float_to_half(float f) {
    const uint32_t x = as_uint(f);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t mag = x & 0x7fffffffu;
    if (mag >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (mag > 0x7f800000u ? 0x200u : 0u));
    if (mag >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (mag < 0x38800000u) {
        const uint32_t q = (uint32_t)std::nearbyint(as_float(mag) * 16777216.0f);
        return (uint16_t)(sign | q);
    }
    uint32_t h = (mag - 0x38000000u) >> 13;
    const uint32_t rem = mag & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

// ---- frames (utils/frame.slang) ----------------------------------------------------------------
template <class R> struct Frame {
    V3<R> t, b, n; // rows of the basis
    V3<R> to_local(V3<R> v) const { return mk(dot(t, v), dot(b, v), dot(n, v)); }
    // frame_to_world = mul(v, basis) = v.x*t + v.y*b + v.z*n
    V3<R> to_world(V3<R> v) const {
        return mk(v.x * t.x + v.y * b.x + v.z * n.x, v.x * t.y + v.y * b.y + v.z * n.y,
                  v.x * t.z + v.y * b.z + v.z * n.z);
    }
};
// make_frame, Duff et al. 2017 (frame.slang:7-13)
template <class R> inline Frame<R> frame_from_normal(V3<R> z) {
    const R sgn = (z.z >= R(0)) ? R(1) : R(-1);
    const R a = R(-1) / (sgn + z.z);
    const R b = z.x * z.y * a;
    Frame<R> f;
    f.t = mk(R(1) + sgn * z.x * z.x * a, sgn * b, -sgn * z.x);
    f.b = mk(b, sgn + z.y * z.y * a, -z.y);
    f.n = z;
    return f;
}
// OrthonormalFrame(n, tangent, handedness) (frame.slang:90-95)
template <class R> inline Frame<R> frame_from_tangent(V3<R> n, V3<R> tg, R hand) {
    const V3<R> N = normalize(n);
    const V3<R> T = normalize(tg - N * dot(tg, N));
    Frame<R> f;
    f.t = T;
    f.b = cross(N, T) * hand;
    f.n = N;
    return f;
}
// apply_normal_map (frame.slang:126-134)
template <class R> inline Frame<R> apply_normal_map(const Frame<R>& f, V3<R> n_local) {
    const V3<R> nN = f.to_world(n_local);
    const V3<R> oT = f.t;
    const V3<R> nT = normalize(oT - nN * dot(oT, nN));
    Frame<R> r;
    r.t = nT;
    r.b = cross(nN, nT);
    r.n = nN;
    return r;
}

// ---- camera (scene/camera.slang:29-56) ----------------------------------------------------------
template <class R> struct Ray {
    V3<R> o, d;
    R tmin, tmax;
};
template <class R> inline Ray<R> camera_ray(const gbpt_camera& c, uint32_t px, uint32_t py,
                                            uint32_t w, uint32_t h) {
    // pixel_to_ndc: p = (pixel + 0.5 + jitter) / dim; ndc = (2,-2) * p + (-1, 1)
    const R x = ((R)px + R(0.5) + (R)c.jitter[0]) / (R)w;
    const R y = ((R)py + R(0.5) + (R)c.jitter[1]) / (R)h;
    const R nx = R(2) * x + R(-1);
    const R ny = R(-2) * y + R(1);
    const V3<R> U = mk<R>(c.U[0], c.U[1], c.U[2]), V = mk<R>(c.V[0], c.V[1], c.V[2]),
                W = mk<R>(c.W[0], c.W[1], c.W[2]);
    Ray<R> r;
    r.o = mk<R>(c.position[0], c.position[1], c.position[2]);
    r.d = normalize((nx * U + ny * V) + W);
    const R inv_cos = R(1) / dot(normalize(W), r.d);
    r.tmin = (R)c.near_plane * inv_cos;
    r.tmax = (R)c.far_plane * inv_cos;
    return r;
}

// offset_ray_origin, Waechter & Binder (scene/hit.slang:14-23), on float32 bits
template <class R> inline V3<R> offset_ray_origin(V3<R> pos, V3<R> n) {
    const float p[3] = {(float)pos.x, (float)pos.y, (float)pos.z};
    const float nn[3] = {(float)n.x, (float)n.y, (float)n.z};
    float out[3];
    for (int a = 0; a < 3; ++a) {
        const int32_t io = (int32_t)(nn[a] * 256.0f);
        const int32_t bits = (int32_t)as_uint(p[a]);
        const float ip = as_float((uint32_t)(bits + (p[a] < 0.0f ? -io : io)));
        out[a] = std::fabs(p[a]) < (1.0f / 16.0f) ? p[a] + nn[a] * (1.0f / 65536.0f) : ip;
    }
    return mk<R>(out[0], out[1], out[2]);
}

// ---- Fresnel (utils/fresnel.slang:14-42) --------------------------------------------------------
template <class R> inline R schlick_term(R cos_theta) {
    return std::pow(maxr(R(1) - cos_theta, R(0)), R(5));
}
template <class R> inline R fresnel_dielectric(R cos_i, R eta) {
    const R sin2_t = eta * eta * (R(1) - cos_i * cos_i);
    if (sin2_t >= R(1)) return R(1);
    const R cos_t = std::sqrt(R(1) - sin2_t);
    const R r_parl = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const R r_perp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return R(0.5) * (r_parl * r_parl + r_perp * r_perp);
}
// reflect2 (utils/math.slang:93-109)
template <class R> inline V3<R> reflect2(V3<R> i, V3<R> n, R ndoti) { return (R(2) * ndoti) * n - i; }
// HLSL refract(i, n, eta)
template <class R> inline V3<R> refract(V3<R> i, V3<R> n, R eta) {
    const R ni = dot(n, i);
    const R k = R(1) - eta * eta * (R(1) - ni * ni);
    if (k < R(0)) return mk(R(0), R(0), R(0));
    return eta * i - (eta * ni + std::sqrt(k)) * n;
}

// ---- GGX (shading/bsdfs/brdf-ggx.slang) ---------------------------------------------------------
template <class R> inline R smith_g1_over_widotn_s(R widotn, R a2) {
    return R(2) / (widotn + std::sqrt(a2 + ((R(1) - a2) * (widotn * widotn))));
}
template <class R> inline R smith_g2_over_widotn_s(R wodotn, R widotn, R a2) {
    const R g1 = widotn * std::sqrt(a2 + ((R(1) - a2) * (wodotn * wodotn)));
    const R g2 = wodotn * std::sqrt(a2 + ((R(1) - a2) * (widotn * widotn)));
    return (R(2) * wodotn) / (g1 + g2);
}
template <class R> inline R smith_g1_over_widotn_v(V3<R> wi, R ax, R ay) {
    return R(2) / (wi.z + length(mk(ax * wi.x, ay * wi.y, wi.z)));
}
template <class R> inline R smith_g2_over_widotn_v(V3<R> wo, V3<R> wi, R ax, R ay) {
    const R g1 = wi.z * length(mk(ax * wo.x, ay * wo.y, wo.z));
    const R g2 = wo.z * length(mk(ax * wi.x, ay * wi.y, wi.z));
    return (R(2) * wo.z) / (g1 + g2);
}
template <class R> inline R ggx_ndf_s(R ndoth2, R a2) {
    return a2 / (C<R>::PI * pow2((ndoth2 * a2) + (R(1) - ndoth2)));
}
template <class R> inline R ggx_ndf_v(V3<R> h, R ax, R ay) {
    const R axy = ax * ay;
    const V3<R> v = mk(ay * h.x, ax * h.y, axy * h.z);
    const R w2 = axy / dot(v, v);
    return axy * w2 * w2 / C<R>::PI;
}
// ggx_VNDF_sample_H, Dupuy & Benyoub 2023 (brdf-ggx.slang:137-152); mad() taken as fma
template <class R> inline V3<R> ggx_vndf_sample_h(V3<R> wi, R ax, R ay, R r0, R r1) {
    const V3<R> wi_std = normalize(mk(wi.x * ax, wi.y * ay, wi.z));
    const R phi = ((R(2) * r0) - R(1)) * C<R>::PI;
    const R z = std::fma(R(1) - r1, R(1) + wi_std.z, -wi_std.z);
    const R sin_theta = std::sqrt(clampr(R(1) - (z * z), R(0), R(1)));
    const R x = sin_theta * std::cos(phi);
    const R y = sin_theta * std::sin(phi);
    const V3<R> wm_std = mk(x, y, z) + wi_std;
    return normalize(mk(wm_std.x * ax, wm_std.y * ay, wm_std.z));
}
template <class R> inline R ggx_vndf_pdf_wo_v(V3<R> wi, V3<R> h, R ax, R ay) {
    return (ggx_ndf_v(h, ax, ay) * smith_g1_over_widotn_v(wi, ax, ay)) / R(4);
}
template <class R> inline R ggx_vndf_pdf_wo_s(R widotn, R ndoth2, R a2) {
    return (ggx_ndf_s(ndoth2, a2) * smith_g1_over_widotn_s(widotn, a2)) / R(4);
}
template <class R> inline R ggx_vndf_h_pdf(V3<R> wi, V3<R> h, R a2) {
    return ggx_ndf_s(pow2(h.z), a2) * smith_g1_over_widotn_s(wi.z, a2) * maxr(R(0), dot(wi, h));
}

template <class R> struct Sample {
    V3<R> wo;
    R pdf;
    V3<R> weight;
    bool valid;
};
template <class R> inline Sample<R> none() {
    Sample<R> s{};
    s.valid = false;
    return s;
}
template <class R> inline Sample<R> some(V3<R> wo, R pdf, V3<R> w) { return {wo, pdf, w, true}; }

static constexpr float BSDF_MIN_COS = 1e-6f; // bsdf.slang:13

// LambertDiffuseBRDF (brdf-lambert-diffuse.slang:32-90); sample_cos (utils/sampling.slang:24-29)
// Directional albedo fit of GGX with the height-correlated Smith G2 (ggx_integral_approx_ and
// ggx_integral_approx_correlated, brdf-ggx.slang:285-316): bias and scale as ratios of polynomials
// in (cos theta, alpha), the bias suppressed for F0 near 0. Matrix rows as the reference writes
// them (float2x2 / float3x3 are row-major; mul(M, x) = rows . x).
template <class R> inline V3<R> ggx_preintegrated(V3<R> F0, R alpha, R cos_theta) {
    const R c = std::fabs(cos_theta);
    const R X[4] = {R(1), c, c * c, c * c * c};
    const R Y[4] = {R(1), alpha, alpha * alpha, alpha * alpha * alpha};
    const R M1[2][2] = {{R(0.995367f), R(-1.38839f)}, {R(-0.24751f), R(1.97442f)}};
    const R M2[3][3] = {{R(1.0f), R(2.68132f), R(52.366f)},
                        {R(16.0932f), R(-3.98452f), R(59.3013f)},
                        {R(-5.18731f), R(255.259f), R(2544.07f)}};
    const R M3[2][2] = {{R(-0.0564526f), R(3.82901f)}, {R(16.91f), R(-11.0303f)}};
    const R M4[3][3] = {{R(1.0f), R(4.11118f), R(-1.37886f)},
                        {R(19.3254f), R(-28.9947f), R(16.9514f)},
                        {R(0.545386f), R(96.0994f), R(-79.4492f)}};
    const R xyw[3] = {X[0], X[1], X[3]}, xzw[3] = {X[0], X[2], X[3]}, Yxyw[3] = {Y[0], Y[1], Y[3]};
    R n1 = 0, d1 = 0, n2 = 0, d2 = 0;
    for (int i = 0; i < 2; ++i) {
        n1 += (M1[i][0] * X[0] + M1[i][1] * X[1]) * Y[i];
        n2 += (M3[i][0] * X[0] + M3[i][1] * X[1]) * Y[i];
    }
    for (int i = 0; i < 3; ++i) {
        d1 += (M2[i][0] * xyw[0] + M2[i][1] * xyw[1] + M2[i][2] * xyw[2]) * Yxyw[i];
        d2 += (M4[i][0] * xzw[0] + M4[i][1] * xzw[1] + M4[i][2] * xzw[2]) * Yxyw[i];
    }
    R bias = n1 / d1;
    const R scale = n2 / d2;
    const R luma = (F0.x + F0.y + F0.z) * (R(1) / R(3));
    bias *= clampr(luma * R(50), R(0), R(1));
    const R sc = maxr(R(0), scale), b = maxr(R(0), bias);
    return mk(F0.x * sc + b, F0.y * sc + b, F0.z * sc + b);
}

template <class R> struct Lambert {
    V3<R> albedo;
    V3<R> get_albedo(V3<R>) const { return albedo; } // brdf-lambert-diffuse.slang:50-52
    template <class G> Sample<R> sample_eval(V3<R> wi, G& rng) const {
        const R x0 = rng.next_float(), x1 = rng.next_float();
        const R su = std::sqrt(x0);
        const V3<R> wo = mk(su * std::cos(C<R>::TWO_PI * x1), su * std::sin(C<R>::TWO_PI * x1),
                            std::sqrt(R(1) - x0));
        if (minr(wi.z, wo.z) < R(BSDF_MIN_COS)) return none<R>();
        return some(wo, C<R>::INV_PI * wo.z, albedo);
    }
    V3<R> eval(V3<R> wi, V3<R> wo) const {
        if (minr(wi.z, wo.z) < R(BSDF_MIN_COS)) return mk(R(0), R(0), R(0));
        return (C<R>::INV_PI * albedo) * wo.z;
    }
    R pdf(V3<R> wi, V3<R> wo) const {
        if (minr(wi.z, wo.z) < R(BSDF_MIN_COS)) return R(0);
        return C<R>::INV_PI * wo.z;
    }
};

// GGXBRDF (brdf-ggx.slang:331-397)
template <class R> struct GGX {
    R ax, ay;
    // brdf-ggx.slang:399-406: the isotropic fit at sqrt(ax ay)
    V3<R> preintegrated(V3<R> F0, V3<R> wi) const {
        return ggx_preintegrated(F0, std::sqrt(ax * ay), wi.z);
    }
    template <class G> Sample<R> sample_eval(V3<R> wi, G& rng) const {
        if (wi.z < R(BSDF_MIN_COS)) return none<R>();
        const R r0 = rng.next_float(), r1 = rng.next_float();
        const V3<R> h = ggx_vndf_sample_h(wi, ax, ay, r0, r1);
        const V3<R> wo = reflect2(wi, h, dot(wi, h));
        if (wo.z < R(BSDF_MIN_COS)) return none<R>();
        const R pdf = ggx_vndf_pdf_wo_v(wi, h, ax, ay);
        const R w = smith_g2_over_widotn_v(wo, wi, ax, ay) / smith_g1_over_widotn_v(wi, ax, ay);
        return some(wo, pdf, mk(w, w, w));
    }
    V3<R> eval(V3<R> wi, V3<R> wo) const {
        if (minr(wi.z, wo.z) < R(BSDF_MIN_COS)) return mk(R(0), R(0), R(0));
        const V3<R> h = normalize(wo + wi);
        const R g2 = smith_g2_over_widotn_v(wo, wi, ax, ay);
        const R d = ggx_ndf_v(h, ax, ay);
        const R v = (d * g2) / R(4);
        return mk(v, v, v);
    }
    R pdf(V3<R> wi, V3<R> wo) const {
        if (minr(wi.z, wo.z) < R(BSDF_MIN_COS)) return R(0);
        const V3<R> h = normalize(wi + wo);
        return ggx_vndf_pdf_wo_v(wi, h, ax, ay);
    }
};

// ConductorFresnelBSDF<GGXBRDF> (bsdf-conductor-fresnel.slang:6-37)
template <class R> struct Conductor {
    GGX<R> ggx;
    V3<R> f0;
    V3<R> get_albedo(V3<R> wi) const { return ggx.preintegrated(f0, wi); } // :39-41
    V3<R> schlick(R c) const {
        const R t = schlick_term(c);
        return f0 + (mk(R(1), R(1), R(1)) - f0) * t;
    }
    template <class G> Sample<R> sample_eval(V3<R> wi, G& rng) const {
        Sample<R> s = ggx.sample_eval(wi, rng);
        if (!s.valid) return s;
        const V3<R> h = normalize(wi + s.wo);
        s.weight = s.weight * schlick(dot(wi, h));
        return s;
    }
    V3<R> eval(V3<R> wi, V3<R> wo) const {
        const V3<R> h = normalize(wi + wo);
        return schlick(dot(wi, h)) * ggx.eval(wi, wo);
    }
    R pdf(V3<R> wi, V3<R> wo) const { return ggx.pdf(wi, wo); }
};

// RoughDielectricBSDF (bsdf-rough-dielectric.slang:65-161)
template <class R> struct RoughDielectric {
    R alpha, eta;
    V3<R> tint;
    // bsdf-rough-dielectric.slang:111-115
    V3<R> get_albedo(V3<R> wi) const {
        const R f = pow2((R(1) - eta) / (R(1) + eta));
        const V3<R> spec = GGX<R>{alpha, alpha}.preintegrated(mk(f, f, f), wi);
        const V3<R> one = mk(R(1), R(1), R(1));
        return spec + (one - spec) * (pow2(eta) * tint);
    }
    template <class G> Sample<R> sample_eval(V3<R> wi, G& rng) const {
        if (wi.z < R(BSDF_MIN_COS)) return none<R>();
        const R a2 = pow2(alpha);
        const R r0 = rng.next_float(), r1 = rng.next_float();
        const V3<R> wm = ggx_vndf_sample_h(wi, alpha, alpha, r0, r1);
        const R widoth = dot(wi, wm);
        const R Rf = fresnel_dielectric(std::fabs(widoth), eta);
        if ((R)rng.next_float() < Rf) {
            const V3<R> wo = reflect2(wi, wm, widoth);
            if (wo.z < R(BSDF_MIN_COS)) return none<R>();
            const R w = smith_g2_over_widotn_s(wo.z, wi.z, a2) / smith_g1_over_widotn_s(wi.z, a2);
            const R pdf = Rf * ggx_vndf_pdf_wo_s(wi.z, pow2(wm.z), a2);
            return some(wo, pdf, mk(w, w, w));
        }
        const V3<R> wo = refract(-wi, wm, eta);
        if ((wo.x == R(0) && wo.y == R(0) && wo.z == R(0)) || wo.z > -R(BSDF_MIN_COS))
            return none<R>();
        const R wodoth = dot(wo, wm);
        const R denom = wodoth + eta * widoth;
        const R pdf = index_matched()
                          ? R(INFINITY)
                          : (R(1) - Rf) * ggx_vndf_h_pdf(wi, wm, a2) * std::fabs(wodoth) / pow2(denom);
        const R w = pow2(eta) * smith_g2_over_widotn_s(std::fabs(wo.z), wi.z, a2) /
                    smith_g1_over_widotn_s(wi.z, a2);
        return some(wo, pdf, tint * w);
    }
    V3<R> eval(V3<R> wi, V3<R> wo) const {
        if (wi.z < R(BSDF_MIN_COS)) return mk(R(0), R(0), R(0));
        if (wo.z > R(BSDF_MIN_COS)) {
            const V3<R> h = normalize(wi + wo);
            const R Rf = fresnel_dielectric(std::fabs(dot(wi, h)), eta);
            return Rf * GGX<R>{alpha, alpha}.eval(wi, wo);
        }
        if (wo.z < -R(BSDF_MIN_COS) && !index_matched()) {
            V3<R> h = normalize(wo + wi * eta);
            h = h * signr(h.z);
            // only a microfacet that wi sees from its front and wo leaves through its back
            // refracts wi into wo; the reference's formula also counts the other side, which
            // the sampler never produces (evaluation must match sample_eval for NEE and MIS)
            if (!(dot(wi, h) > R(0) && dot(wo, h) < R(0))) return mk(R(0), R(0), R(0));
            const R Rf = fresnel_dielectric(std::fabs(dot(wi, h)), eta);
            return (R(1) - Rf) * btdf_eval(wi, wo);
        }
        // Index-matched boundary (|eta - 1| < 1e-3; the IOR bookkeeping lands on 0.99999994 as
        // often as on 1): every microfacet refracts (nearly) straight through, a delta lobe that
        // only sample_eval produces (it reports pdf = inf). The microfacet formula would give a
        // density the sampler never draws, so evaluation (next-event estimation, MIS) sees no
        // transmission lobe there.
        return mk(R(0), R(0), R(0));
    }
    bool index_matched() const { return std::fabs(eta - R(1)) < R(1e-3); }
    // GGXBTDF::eval (brdf-ggx.slang:427-444)
    V3<R> btdf_eval(V3<R> wi, V3<R> wo) const {
        if ((wi.z < R(BSDF_MIN_COS)) || (wo.z > -R(BSDF_MIN_COS))) return mk(R(0), R(0), R(0));
        V3<R> h = normalize(wo + (wi * eta));
        h = h * signr(h.z);
        const R widoth = dot(wi, h), wodoth = dot(wo, h);
        const R a2 = pow2(alpha);
        const R g2 = smith_g2_over_widotn_s(std::fabs(wo.z), wi.z, a2);
        const R d = ggx_ndf_s(pow2(h.z), a2);
        const R denom = wodoth + (eta * widoth);
        const R jac = pow2(eta) * widoth * wodoth / pow2(denom);
        return tint * (d * g2 * std::fabs(jac));
    }
    R pdf(V3<R> wi, V3<R> wo) const {
        if (wi.z < R(BSDF_MIN_COS)) return R(0);
        const R a2 = pow2(alpha);
        if (wo.z > R(BSDF_MIN_COS)) {
            const V3<R> h = normalize(wi + wo);
            const R Rf = fresnel_dielectric(std::fabs(dot(wi, h)), eta);
            return Rf * ggx_vndf_pdf_wo_s(wi.z, pow2(maxr(R(0), h.z)), a2);
        }
        if (wo.z < -R(BSDF_MIN_COS) && !index_matched()) { // else a delta transmission
            V3<R> h = normalize(wo + wi * eta);
            h = h * signr(h.z);
            if (!(dot(wi, h) > R(0) && dot(wo, h) < R(0))) return R(0); // as eval()
            const R Rf = fresnel_dielectric(std::fabs(dot(wi, h)), eta);
            const R wodoth = dot(wo, h);
            const R denom = wodoth + eta * dot(wi, h);
            return (R(1) - Rf) * ggx_vndf_h_pdf(wi, h, a2) * std::fabs(wodoth) / pow2(denom);
        }
        return R(0);
    }
};

// FresnelMixBSDF<GGX, Lambert> (bsdf-fresnel-mix.slang:7-63)
template <class R> struct OpaqueDielectric {
    GGX<R> layer;
    Lambert<R> base;
    R f0;
    // bsdf-fresnel-mix.slang:50-53
    V3<R> get_albedo(V3<R> wi) const {
        const V3<R> spec = layer.preintegrated(mk(f0, f0, f0), wi);
        return spec + (mk(R(1), R(1), R(1)) - spec) * base.get_albedo(wi);
    }
    R F(R c) const { return f0 + (R(1) - f0) * schlick_term(c); }
    V3<R> eval(V3<R> wi, V3<R> wo) const {
        const V3<R> h = normalize(wi + wo);
        const R f = F(dot(wi, h));
        return lerp(base.eval(wi, wo), layer.eval(wi, wo), f);
    }
    R pdf(V3<R> wi, V3<R> wo) const {
        const R f = F(wi.z);
        return lerp(base.pdf(wi, wo), layer.pdf(wi, wo), f);
    }
    template <class G> Sample<R> sample_eval(V3<R> wi, G& rng) const {
        const R f = F(wi.z);
        const Sample<R> s =
            (R)rng.next_float() < f ? layer.sample_eval(wi, rng) : base.sample_eval(wi, rng);
        if (!s.valid) return s;
        const R p = pdf(wi, s.wo);
        return some(s.wo, p, eval(wi, s.wo) / p);
    }
};

// MixBSDF (bsdf-mix.slang:7-49); the draw is skipped when weight == 0 (`weight > 0.0f &&`).
// A weight of exactly 0 or 1 is evaluated exactly: lerp(x, y, 1) = y and the sampled lobe's
// (weight * pdf) / pdf = weight. Rounded, that round trip turns the unbounded pdf of an
// index-matched refraction (relative IOR 1, denominator wo.h + eta wi.h = 0) into NaN.
template <class R, class B0, class B1> struct Mix {
    B0 b0;
    B1 b1;
    R w;
    // bsdf-mix.slang:51-54 (a plain lerp, also at weight 0 and 1)
    V3<R> get_albedo(V3<R> wi) const { return lerp(b0.get_albedo(wi), b1.get_albedo(wi), w); }
    V3<R> eval(V3<R> wi, V3<R> wo) const {
        if (w == R(0)) return b0.eval(wi, wo);
        if (w == R(1)) return b1.eval(wi, wo);
        return lerp(b0.eval(wi, wo), b1.eval(wi, wo), w);
    }
    R pdf(V3<R> wi, V3<R> wo) const {
        if (w == R(0)) return b0.pdf(wi, wo);
        if (w == R(1)) return b1.pdf(wi, wo);
        return lerp(b0.pdf(wi, wo), b1.pdf(wi, wo), w);
    }
    template <class G> Sample<R> sample_eval(V3<R> wi, G& rng) const {
        if (w > R(0) && (R)rng.next_float() < w) {
            const Sample<R> s = b1.sample_eval(wi, rng);
            // a delta sample (pdf = inf) passes through: w f1 / (w p1) = its own weight
            if (!s.valid || w == R(1) || !(s.pdf < R(INFINITY))) return s;
            const R mp = lerp(b0.pdf(wi, s.wo), s.pdf, w);
            const V3<R> me = lerp(b0.eval(wi, s.wo), s.weight * s.pdf, w);
            return some(s.wo, mp, me / mp);
        }
        const Sample<R> s = b0.sample_eval(wi, rng);
        if (!s.valid || w == R(0) || !(s.pdf < R(INFINITY))) return s;
        const R mp = lerp(s.pdf, b1.pdf(wi, s.wo), w);
        const V3<R> me = lerp(s.weight * s.pdf, b1.eval(wi, s.wo), w);
        return some(s.wo, mp, me / mp);
    }
};

template <class R> using Dielectric = Mix<R, OpaqueDielectric<R>, RoughDielectric<R>>;
template <class R> using Substrate = Mix<R, Dielectric<R>, Conductor<R>>;

// Per-shading-point material instance: DiffuseMaterial (diffuse-material.slang:7-43) or the
// OpenPBR substrate (openpbr-material.slang:220-323). The clear-coat and sheen lobes of
// OpenPBRMaterial are compile-time absent for these models (weights folded to 0), so
// OpenPBRBSDF reduces to its substrate.
template <class R> struct MaterialBSDF {
    bool diffuse;
    Lambert<R> lambert;
    Substrate<R> substrate;
    R eta; // interior relative IOR (1 for opaque models)
    template <class G> Sample<R> sample_eval(V3<R> wi, G& rng) const {
        return diffuse ? lambert.sample_eval(wi, rng) : substrate.sample_eval(wi, rng);
    }
    V3<R> eval(V3<R> wi, V3<R> wo) const {
        return diffuse ? lambert.eval(wi, wo) : substrate.eval(wi, wo);
    }
    R pdf(V3<R> wi, V3<R> wo) const { return diffuse ? lambert.pdf(wi, wo) : substrate.pdf(wi, wo); }
    V3<R> get_albedo(V3<R> wi) const {
        return diffuse ? lambert.get_albedo(wi) : substrate.get_albedo(wi);
    }
};

static constexpr float MIN_ROUGHNESS = 0.0316f; // material.slang:23

// OpenPBRMaterial::get_sample for the configured models; `ior` is the RenderContext IOR and
// `front_facing` the ShadingData flag.
template <class R> inline MaterialBSDF<R> make_material(const gbpt_material& m, V3<R> base_tex,
                                                        R ior, bool front_facing) {
    MaterialBSDF<R> mb{};
    const V3<R> base = mk<R>(m.base_color[0], m.base_color[1], m.base_color[2]) * base_tex;
    if (m.model == GBPT_MATERIAL_DIFFUSE) {
        mb.diffuse = true;
        mb.lambert.albedo = base;
        mb.eta = R(1);
        return mb;
    }
    mb.diffuse = false;
    const float min_alpha_f = MIN_ROUGHNESS * MIN_ROUGHNESS; // ggx_roughness_to_alpha in float
    const R min_alpha = (R)min_alpha_f;
    const R ax = maxr((R)m.specular_alpha[0], min_alpha);
    const R ay = maxr((R)m.specular_alpha[1], min_alpha);
    const R sior = (R)m.specular_ior;
    const R ior_t = (sior - R(1)) / (sior + R(1));
    const R f0 = clampr((R)m.specular_weight * ior_t * ior_t, R(0), R(1));
    R eta = R(1), tw = R(0);
    V3<R> tcol = mk(R(1), R(1), R(1));
    const bool transmission = m.model == GBPT_MATERIAL_OPENPBR_TRANSMISSION;
    if (transmission) {
        eta = ior / (front_facing ? sior : R(1));
        tw = (R)m.transmission_weight;
        tcol = mk<R>(m.transmission_color[0], m.transmission_color[1], m.transmission_color[2]);
    }
    const R alpha_iso = transmission ? std::sqrt(ax * ay) : ax;
    mb.substrate.b0.b0.layer = GGX<R>{ax, ay};
    mb.substrate.b0.b0.base = Lambert<R>{base};
    mb.substrate.b0.b0.f0 = f0;
    mb.substrate.b0.b1 = RoughDielectric<R>{alpha_iso, eta, tcol};
    mb.substrate.b0.w = tw;
    mb.substrate.b1.ggx = GGX<R>{ax, ay};
    mb.substrate.b1.f0 = base;
    mb.substrate.w = (R)m.metalness;
    mb.eta = eta;
    return mb;
}

// Power-heuristic weight of a strategy with density a against one with density b, written as
// 1 / (1 + (b/a)^2) so an unbounded a (a near-delta lobe) gives 1 instead of inf/inf.
template <class R> inline R power_heuristic(R a, R b) {
    if (!(a > R(0))) return R(0);
    const R r = b / a;
    return R(1) / (R(1) + r * r);
}

// yuv_luminance (colors/colorspace_yuv.slang:5-7)
template <class R> inline R yuv_luminance(V3<R> c) {
    return dot(c, mk(R(0.299f), R(0.587f), R(0.114f)));
}

} // namespace oracle

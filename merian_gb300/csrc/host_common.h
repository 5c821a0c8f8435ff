// Host-side helpers shared by the scene generators, the BVH builder and the C ABI.
#pragma once

#include "gbpt.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

namespace gbpt {

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalize(V3 a) {
    const float l = std::sqrt(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}

// Octahedral projection + packSnorm2x16 (merian encoding.slang:14-30). packSnorm2x16 rounds
// clamp(v,-1,1)*32767 to nearest (ties away from zero) and stores x in the low 16 bits.
inline uint32_t encode_normal(V3 n) {
    const float inv_l1 = 1.0f / ((std::fabs(n.x) + std::fabs(n.y)) + std::fabs(n.z));
    float px, py;
    if (n.z < 0.0f) {
        px = std::copysign(1.0f - std::fabs(n.y * inv_l1), n.x);
        py = std::copysign(1.0f - std::fabs(n.x * inv_l1), n.y);
    } else {
        px = n.x * inv_l1;
        py = n.y * inv_l1;
    }
    auto pack = [](float v) -> uint32_t {
        v = v < -1.0f ? -1.0f : (v > 1.0f ? 1.0f : v);
        const int32_t i = (int32_t)std::round(v * 32767.0f);
        return (uint32_t)(uint16_t)(int16_t)i;
    };
    return pack(px) | (pack(py) << 16);
}

// float -> IEEE binary16, round to nearest even (Slang half(x) conversion).
inline uint16_t float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t mag = x & 0x7fffffffu;
    if (mag >= 0x7f800000u) { // inf / nan
        return (uint16_t)(sign | 0x7c00u | (mag > 0x7f800000u ? 0x200u : 0u));
    }
    if (mag >= 0x477ff000u) { // rounds to >= 65520 -> inf
        return (uint16_t)(sign | 0x7c00u);
    }
    if (mag < 0x38800000u) { // half subnormal (or zero): value = q * 2^-24
        float a;
        std::memcpy(&a, &mag, 4);
        // exact power-of-two scaling, then round half to even; q = 1024 is the smallest normal
        const uint32_t q = (uint32_t)std::nearbyint(a * 16777216.0f);
        return (uint16_t)(sign | q);
    }
    // normal: rebias exponent 127 -> 15, keep 10 mantissa bits
    uint32_t h = ((mag - 0x38000000u) >> 13);
    const uint32_t rem = mag & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

inline uint32_t pack_half2(float a, float b) {
    return (uint32_t)float_to_half(a) | ((uint32_t)float_to_half(b) << 16);
}

// PCG32 (O'Neill, pcg-random.org): 64-bit LCG state, XSH-RR output. Integer-only, so a seed
// gives the same stream on every host.
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    Pcg32(uint64_t seed, uint64_t stream) {
        inc = (stream << 1u) | 1u;
        next();
        state += seed;
        next();
    }
    uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // [0, 1) with 24 random bits
    float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
    double uniform_d() {
        const uint64_t hi = next() >> 5, lo = next() >> 6;
        return ((double)hi * 67108864.0 + (double)lo) * (1.0 / 9007199254740992.0);
    }
};

// Deterministic double-precision exp / log / sin / cos for the scene generators: range reduction
// plus truncated Taylor / atanh series using only IEEE +, -, *, / and exact power-of-two scaling,
// so every host (any libm, any FMA policy; this code is built with -ffp-contract=off) produces
// the same bits. Accurate to a few 1e-16 relative, which is all the generators need.
namespace det {
constexpr double kLn2Hi = 6.93147180369123816490e-01; // ln 2 split so n*kLn2Hi is exact
constexpr double kLn2Lo = 1.90821492927058770002e-10;
constexpr double kPi = 3.14159265358979323846;
inline double exp(double x) {
    if (x > 700.0) x = 700.0;
    if (x < -700.0) return 0.0;
    const double n = std::floor(x / 0.69314718055994530942 + 0.5);
    const double r = (x - n * kLn2Hi) - n * kLn2Lo; // |r| <= ln2/2
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 20; ++k) {
        term = term * r / (double)k;
        sum = sum + term;
    }
    return std::ldexp(sum, (int)n);
}
inline double log(double x) { // x > 0
    int e = 0;
    double m = std::frexp(x, &e); // x = m 2^e, m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0); // |s| < 0.172
    const double s2 = s * s;
    double term = s, sum = s;
    for (int k = 3; k <= 41; k += 2) {
        term = term * s2;
        sum = sum + term / (double)k;
    }
    return 2.0 * sum + (double)e * kLn2Hi + (double)e * kLn2Lo;
}
inline void sincos(double x, double& s, double& c) {
    // reduce to [-pi/4, pi/4] by quarter turns
    const double q = std::floor(x / (kPi * 0.5) + 0.5);
    const double r = x - q * (kPi * 0.5);
    const double r2 = r * r;
    double ts = r, ss = r, tc = 1.0, sc = 1.0;
    for (int k = 1; k <= 12; ++k) {
        ts = -ts * r2 / (double)((2 * k) * (2 * k + 1));
        ss = ss + ts;
        tc = -tc * r2 / (double)((2 * k - 1) * (2 * k));
        sc = sc + tc;
    }
    const long long qi = ((long long)q % 4 + 4) % 4;
    if (qi == 0) { s = ss; c = sc; }
    else if (qi == 1) { s = sc; c = -ss; }
    else if (qi == 2) { s = -ss; c = -sc; }
    else { s = -sc; c = ss; }
}
} // namespace det

void set_error(const std::string& msg);

// PNG to RGBA8, top row first (png.cpp).
bool decode_png(const uint8_t* data, size_t size, std::vector<uint8_t>& rgba, uint32_t& width,
                uint32_t& height, std::string& err);
bool read_png_file(const std::string& path, std::vector<uint8_t>& rgba, uint32_t& width,
                   uint32_t& height, std::string& err);

// ---- CWBVH (compressed 8-wide BVH, Ylitie/Karras/Laine HPG 2017 layout) -------------------
// Node = 5 x 16 bytes:
//   w0: p.x p.y p.z (float), e.x | e.y<<8 | e.z<<16 | imask<<24
//   w1: child_base, tri_base, meta[0..3], meta[4..7]
//   w2: q_lo.x[0..7], q_lo.y[0..7]   (bytes)
//   w3: q_lo.z[0..7], q_hi.x[0..7]
//   w4: q_hi.y[0..7], q_hi.z[0..7]
// meta: inner child = 0b001_11sss (24 + slot); leaf = unary triangle count in bits 5..7, triangle
// offset from tri_base in bits 0..4; empty = 0.
struct CwNode {
    uint32_t w[20];
};
static_assert(sizeof(CwNode) == 80, "CWBVH node must be 80 bytes");

// Triangle record used by the traversal: 3 x float4 = 48 bytes
//   (v0.xyz, primitive id bits), (v1.xyz, geometry id bits), (v2.xyz, 0)
struct TriRecord {
    float v0[3];
    uint32_t prim;
    float v1[3];
    uint32_t geom;
    float v2[3];
    uint32_t pad;
};
static_assert(sizeof(TriRecord) == 48, "triangle record must be 48 bytes");

struct BuildInput {
    // world-space triangles
    std::vector<float> v; // 9 floats per triangle
    std::vector<uint32_t> prim;
    std::vector<uint32_t> geom;
    std::vector<uint32_t> flags; // instance mask (bits 0-7), two-sided (bit 8), flip (bit 9)
    // split triangles whose bounding box is loose into clipped references (never for TLAS
    // builds, whose "triangles" are instance boxes): box area above split_ratio x twice the
    // triangle area, at most split_depth halvings
    bool split = false;
    double split_ratio = 2.0;
    int split_depth = 4;
};

struct CwBvh {
    std::vector<CwNode> nodes;
    std::vector<TriRecord> tris;
    uint32_t depth = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

// Binned-SAH BVH2 build, greedy surface-area collapse to 8-wide, octant slot ordering and 8-bit
// conservative quantisation. Returns false (and sets the error) when the tree is deeper than
// max_depth.
bool build_cwbvh(const BuildInput& in, CwBvh& out, uint32_t max_depth);

// Walker's alias table (Vose's construction) of the discrete distribution w[0, n): entry i is
// (the probability that bin i keeps i, as float bits; the bin it gives otherwise). Built in
// double in a fixed order, so every host makes the same table.
inline void alias_table(const double* w, uint32_t n, uint32_t* out) {
    double sum = 0.0;
    for (uint32_t i = 0; i < n; ++i) sum += w[i];
    std::vector<double> q(n);
    std::vector<uint32_t> small, large;
    for (uint32_t i = 0; i < n; ++i) {
        q[i] = sum > 0.0 ? w[i] * (double)n / sum : 1.0;
        (q[i] < 1.0 ? small : large).push_back(i);
    }
    while (!small.empty() && !large.empty()) {
        const uint32_t a = small.back(), b = large.back();
        small.pop_back();
        const float pa = (float)q[a];
        std::memcpy(&out[2 * a], &pa, 4);
        out[2 * a + 1] = b;
        q[b] = (q[b] + q[a]) - 1.0;
        if (q[b] < 1.0) {
            large.pop_back();
            small.push_back(b);
        }
    }
    // what rounding leaves on either list keeps its own bin
    for (const std::vector<uint32_t>* l : {&small, &large})
        for (uint32_t i : *l) {
            const float one = 1.0f;
            std::memcpy(&out[2 * i], &one, 4);
            out[2 * i + 1] = i;
        }
}

} // namespace gbpt

// Device view of a scene in HBM and the CWBVH traversal.
//
// Traversal replaces the hardware ray query merian issues through TraceRayInline with
// RAY_FLAG_CULL_BACK_FACING_TRIANGLES (acceleration-structure.slang:59-72) on ForceOpaque
// instances (scene.cpp:1849-1850). Closest hit over triangles whose instance mask intersects the
// ray mask, back faces culled unless the geometry is TwoSided, the front face swapped by
// FlipFacing (scene.cpp:1841-1848). Ties at equal t go to the smallest (geometry, primitive), so
// the result does not depend on the BVH layout.
#pragma once

#include "device_math.cuh"

#include <type_traits>
#include "gbpt.h"
#include "runtime.h"

namespace gbpt {

struct GeomGPU {
    uint32_t first_vertex, first_triangle, material, flags;
};

// per-triangle flag word (third float4 of a triangle record)
constexpr uint32_t kTriTwoSided = 1u << 8;
constexpr uint32_t kTriFlip = 1u << 9;
constexpr uint32_t kTriAlpha = 1u << 10; // non-opaque geometry: candidate hits run the alpha test

struct DevScene {
    const uint4* __restrict__ nodes;  // 5 per CWBVH node
    const float4* __restrict__ tris;  // 3 per triangle record and copy
    uint32_t tri_stride;              // float4 from one copy of the records to the next
    const uint32_t* __restrict__ verts; // gbpt_packed_vertex as 6 words
    const uint32_t* __restrict__ idx;
    const uint4* __restrict__ tri_verts; // 5 per triangle (3 vertices, padded) or null
    const GeomGPU* __restrict__ geoms;
    const float4* __restrict__ mats;  // gbpt_material as 5 float4
    uint32_t geom_count;
    // environment
    const float4* __restrict__ env;
    uint32_t ew, eh;
    float env_m[9];
    float env_intensity;
    const float* __restrict__ env_marg; // eh + 1, normalised
    const float* __restrict__ env_cond; // eh * (ew + 1), normalised per row
    const float* __restrict__ env_func; // eh * ew
    float env_func_int;
    // emissive triangles
    const float4* __restrict__ light_tris; // 3 per light: v0 (w = geometry), v1, v2
    const float* __restrict__ light_cdf;   // n_lights, inclusive, normalised
    uint32_t n_lights;
    float light_total; // sum of area x luminance
    float p_env;       // probability of choosing the environment in NEE
    // guide tables of the light, marginal and conditional CDFs: entry k is the upper bound of
    // k / G (G a power of two), so the search for u covers [guide[k], guide[k + 1]] only
    const uint32_t* __restrict__ light_guide;
    const uint2* __restrict__ env_rows; // alias tables (GBPT_ENV_ALIAS): per row, per texel
    const uint2* __restrict__ env_cols;
    const uint32_t* __restrict__ env_marg_guide;
    const uint32_t* __restrict__ env_cond_guide; // G + 1 per row
    uint32_t light_g, env_marg_g, env_cond_g;
    // two-level scenes: instance records (7 float4 each), n_inst = 0 for single-level scenes
    const float4* __restrict__ inst;
    uint32_t n_inst;
    // RGBA8 textures: texels of all textures, (first texel, width, height, sRGB) per texture and
    // the sRGB-to-linear table
    const uchar4* __restrict__ tex;
    const uint4* __restrict__ tex_info;
    uint32_t n_tex;
    const float* __restrict__ srgb_lut;
};

struct Hit {
    float t, u, v;
    uint32_t prim, geom; // geom = 0xFFFFFFFF on miss (the scene-global geometry index)
    uint32_t inst;       // instance index of two-level scenes, 0xFFFFFFFF otherwise
};

// ---- alpha test of non-opaque geometry (material-system.slang:28-38, scene.slang:500-519) --------
// The material's alpha texture, bilinear with repeat addressing at level 0, at the candidate hit's
// interpolated uv; alpha below 0.5 (merian_alpha_test_threshold) discards the candidate. Rounded
// operations in a fixed order, shared with the oracle, so the decision is bit-identical.
constexpr float kAlphaThreshold = 0.5f;

GBPT_DI float texture_alpha(const DevScene& sc, uint32_t t, float u, float v) {
    const uint4 info = __ldg(&sc.tex_info[t]);
    const int w = (int)info.y, h = (int)info.z;
    if (!(fabsf(u) < 65536.0f)) u = 0.0f; // half uvs: only NaN / inf are out of range
    if (!(fabsf(v) < 65536.0f)) v = 0.0f;
    const float x = __fsub_rn(__fmul_rn(u, (float)w), 0.5f);
    const float y = __fsub_rn(__fmul_rn(v, (float)h), 0.5f);
    const float fx = floorf(x), fy = floorf(y);
    const float a = __fsub_rn(x, fx), b = __fsub_rn(y, fy);
    const int ix = (int)fx, iy = (int)fy;
    const int x0 = ((ix % w) + w) % w, x1 = (((ix + 1) % w) + w) % w;
    const int y0 = ((iy % h) + h) % h, y1 = (((iy + 1) % h) + h) % h;
    const uchar4* base = sc.tex + info.x;
    auto alpha = [&](int xx, int yy) {
        return __fmul_rn((float)__ldg(&base[(size_t)yy * w + xx]).w, 1.0f / 255.0f);
    };
    const float ia = __fsub_rn(1.0f, a), ib = __fsub_rn(1.0f, b);
    const float top = __fadd_rn(__fmul_rn(alpha(x0, y0), ia), __fmul_rn(alpha(x1, y0), a));
    const float bot = __fadd_rn(__fmul_rn(alpha(x0, y1), ia), __fmul_rn(alpha(x1, y1), a));
    return __fadd_rn(__fmul_rn(top, ib), __fmul_rn(bot, b));
}

// True when the candidate hit (geometry, primitive, barycentrics u, v) is transparent.
GBPT_DI bool alpha_discard(const DevScene& sc, uint32_t geom, uint32_t prim, float bu, float bv) {
    const GeomGPU g = sc.geoms[geom];
    const int tex = __float_as_int(__ldg(&sc.mats[5ull * g.material + 4]).y);
    if (tex < 0 || (uint32_t)tex >= sc.n_tex) return false;
    const uint32_t tri = g.first_triangle + prim;
    float uvx[3], uvy[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t* v =
            sc.tri_verts ? (const uint32_t*)(sc.tri_verts + 5ull * tri) + 6 * k
                         : sc.verts + 6ull * (g.first_vertex + __ldg(&sc.idx[3 * tri + k]));
        const uint32_t uv = __ldg(v + 4);
        uvx[k] = __half2float(__ushort_as_half((unsigned short)(uv & 0xFFFFu)));
        uvy[k] = __half2float(__ushort_as_half((unsigned short)(uv >> 16)));
    }
    const float b0 = __fsub_rn(__fsub_rn(1.0f, bu), bv);
    const float u = __fadd_rn(__fadd_rn(__fmul_rn(b0, uvx[0]), __fmul_rn(bu, uvx[1])),
                              __fmul_rn(bv, uvx[2]));
    const float v = __fadd_rn(__fadd_rn(__fmul_rn(b0, uvy[0]), __fmul_rn(bu, uvy[1])),
                              __fmul_rn(bv, uvy[2]));
    return texture_alpha(sc, (uint32_t)tex, u, v) < kAlphaThreshold;
}

// ---- watertight test (Woop, Benthin, Wald 2013) -------------------------------------------------
// Explicit round-to-nearest intrinsics (no FMA contraction) so the float result equals the
// host oracle's bit for bit.
struct RayPre {
    // the axes kx, ky, kz in bits 0-1, 2-3, 4-5 (kx = kz + 1, ky = kz + 2 mod 3); bit 6 when the
    // direction is negative along kz. The watertight test's paper swaps kx and ky for that sign
    // to keep the winding; keeping one frame per kz negates U, V, W, det and T instead, which
    // leaves t, u and v unchanged and flips the facing. The traversal keeps more of the ray in
    // the same register (set_ray, TraceState): 7 - the direction octant in bits 8-10, the ray's
    // instance mask in bits 16-23 and the stack depth in bits 24-31.
    uint32_t k;
    float Sx, Sy, Sz;
    float ox, oy, oz; // origin permuted to (kx, ky, kz)
    GBPT_DI int kx() const { return (int)(k & 3u); }
    GBPT_DI int ky() const { return (int)((k >> 2) & 3u); }
    GBPT_DI int kz() const { return (int)((k >> 4) & 3u); }
    GBPT_DI uint32_t oct_inv() const { return (k >> 8) & 7u; }
    GBPT_DI uint32_t mask() const { return (k >> 16) & 0xFFu; }
};
GBPT_DI float pick(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }
GBPT_DI RayPre ray_pre(float3 o, float3 d) {
    RayPre p;
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    const int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    const int kx = kz == 2 ? 0 : kz + 1;
    const int ky = kx == 2 ? 0 : kx + 1;
    const float dkz = pick(d.x, d.y, d.z, kz);
    p.k = (uint32_t)kx | ((uint32_t)ky << 2) | ((uint32_t)kz << 4) | (dkz < 0.0f ? 64u : 0u);
    p.Sx = __fdiv_rn(pick(d.x, d.y, d.z, kx), dkz);
    p.Sy = __fdiv_rn(pick(d.x, d.y, d.z, ky), dkz);
    p.Sz = __frcp_rn(dkz);
    p.ox = pick(o.x, o.y, o.z, kx);
    p.oy = pick(o.x, o.y, o.z, ky);
    p.oz = pick(o.x, o.y, o.z, kz);
    return p;
}

// Returns true with t, u, v when hit within [tmin, tmax] on an accepted face.
// With GBPT_DEFER_UV the barycentrics are returned undivided (u_out = V, v_out = W, det_out =
// det): the caller divides them once for the final hit instead of at every accepted candidate.
#ifndef GBPT_DEFER_UV
#define GBPT_DEFER_UV 1
#endif
GBPT_DI bool intersect_tri(const RayPre& p, float4 a4, float4 b4, float4 c4, uint32_t tflags,
                           float tmin, float tmax, float& t_out, float& u_out, float& v_out,
                           float& det_out) {
#if GBPT_TRI_AXIS_COPIES
    // the record copy of axis kz holds the coordinates (kx, ky, kz)
    const float Akx = __fsub_rn(a4.x, p.ox);
    const float Aky = __fsub_rn(a4.y, p.oy);
    const float Akz = __fsub_rn(a4.z, p.oz);
    const float Bkx = __fsub_rn(b4.x, p.ox);
    const float Bky = __fsub_rn(b4.y, p.oy);
    const float Bkz = __fsub_rn(b4.z, p.oz);
    const float Ckx = __fsub_rn(c4.x, p.ox);
    const float Cky = __fsub_rn(c4.y, p.oy);
    const float Ckz = __fsub_rn(c4.z, p.oz);
#else
    const int kx = p.kx(), ky = p.ky(), kz = p.kz();
    const float Akx = __fsub_rn(pick(a4.x, a4.y, a4.z, kx), p.ox);
    const float Aky = __fsub_rn(pick(a4.x, a4.y, a4.z, ky), p.oy);
    const float Akz = __fsub_rn(pick(a4.x, a4.y, a4.z, kz), p.oz);
    const float Bkx = __fsub_rn(pick(b4.x, b4.y, b4.z, kx), p.ox);
    const float Bky = __fsub_rn(pick(b4.x, b4.y, b4.z, ky), p.oy);
    const float Bkz = __fsub_rn(pick(b4.x, b4.y, b4.z, kz), p.oz);
    const float Ckx = __fsub_rn(pick(c4.x, c4.y, c4.z, kx), p.ox);
    const float Cky = __fsub_rn(pick(c4.x, c4.y, c4.z, ky), p.oy);
    const float Ckz = __fsub_rn(pick(c4.x, c4.y, c4.z, kz), p.oz);
#endif
    const float Ax = __fsub_rn(Akx, __fmul_rn(p.Sx, Akz));
    const float Ay = __fsub_rn(Aky, __fmul_rn(p.Sy, Akz));
    const float Bx = __fsub_rn(Bkx, __fmul_rn(p.Sx, Bkz));
    const float By = __fsub_rn(Bky, __fmul_rn(p.Sy, Bkz));
    const float Cx = __fsub_rn(Ckx, __fmul_rn(p.Sx, Ckz));
    const float Cy = __fsub_rn(Cky, __fmul_rn(p.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    if (!(tflags & kTriTwoSided)) {
        const bool front = (det > 0.0f) != ((p.k & 64u) != 0u);
        if (front == ((tflags & kTriFlip) != 0)) return false;
    }
    const float Az = __fmul_rn(p.Sz, Akz);
    const float Bz = __fmul_rn(p.Sz, Bkz);
    const float Cz = __fmul_rn(p.Sz, Ckz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float t = __fdiv_rn(T, det);
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
#if GBPT_DEFER_UV
    u_out = V;
    v_out = W;
    det_out = det;
#else
    u_out = __fdiv_rn(V, det);
    v_out = __fdiv_rn(W, det);
    det_out = 1.0f;
#endif
    return true;
}

// ---- CWBVH traversal ----------------------------------------------------------------------------
// Traversal stack entries per ray. The builder bounds the tree depth (24 levels), which with
// postponed triangle groups and instance entries stays below the default. A build with a smaller
// GBPT_STACK_SIZE makes deep traversals overflow: the overflow sets the kernels' error word
// (GBPT_ERR_DEVICE on the host) and finishes the ray with what it found, never a fault, so the
// error path can be exercised on purpose.
#ifndef GBPT_STACK_SIZE
#define GBPT_STACK_SIZE 48
#endif
constexpr int kStackSize = GBPT_STACK_SIZE;
static_assert(kStackSize >= 1, "the traversal needs a stack entry");
constexpr uint32_t kNoInst = 0xFFFFFFFFu;

// Work of the instrumented traversal (COUNT): nodes visited and triangles tested per lane, and
// on the first active lane of each warp-wide step the step and its active lanes.
struct TraceCounters {
    uint32_t nodes, tris;
    uint32_t node_steps, node_lanes, tri_steps, tri_lanes;
};
GBPT_DI void count_step(uint32_t& steps, uint32_t& lanes) {
    const uint32_t m = __activemask();
    if ((threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) {
        steps++;
        lanes += __popc(m);
    }
}

GBPT_DI float safe_rcp(float d) {
    const float m = 1e-20f;
    return __frcp_rn(fabsf(d) > m ? d : copysignf(m, d));
}

// Instance records of two-level scenes, 7 float4 each: object-to-world rows (0..2), world-to-
// object rows (3..5), then (BLAS root node, mask, first geometry of the BLAS, 0) as bits. The
// transforms are evaluated with explicit round-to-nearest operations in a fixed order, as the
// oracle does, so transformed rays (and therefore hits) are bit-identical to the host's.
GBPT_DI float xform_row(float4 r, float3 p, float w) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r.x, p.x), __fmul_rn(r.y, p.y)),
                               __fmul_rn(r.z, p.z)),
                     __fmul_rn(r.w, w));
}
GBPT_DI float3 xform_point(float4 r0, float4 r1, float4 r2, float3 p) {
    return f3(xform_row(r0, p, 1.0f), xform_row(r1, p, 1.0f), xform_row(r2, p, 1.0f));
}
GBPT_DI float3 xform_vector(float4 r0, float4 r1, float4 r2, float3 v) {
    return f3(xform_row(r0, v, 0.0f), xform_row(r1, v, 0.0f), xform_row(r2, v, 0.0f));
}

// ---- traversal state and loop ------------------------------------------------------------------
// One loop serves the per-thread queries (trace_ray) and the persistent warps (trace_persistent).
// In the persistent form a lane postpones its pending triangle tests (pushes the triangle group
// onto its stack) when fewer than `postpone_lanes` lanes of the warp have triangles to test, so
// node steps and triangle steps stay in lockstep across the warp, and the warp leaves the loop to
// refill idle lanes once fewer than `refill_lanes` lanes are busy (both launch arguments). Two-level scenes: a top-level leaf is an
// instance; entering it pushes what is left of the top level, transforms the ray to object space
// (t is unchanged: the direction is not renormalised) and continues from the BLAS root; when the
// stack drops back to the entry depth the world ray is restored. The closest hit and the tie rule
// (equal t: smallest geometry, primitive, instance) do not depend on the visit order.


struct TraceState {
    const uint4* nodes;  // the ray's scene (rays of one launch may belong to different scenes)
    const float4* tris;  // the records (copy-major layout: the current ray's copy)
    const float4* tris_base; // copy 0 of the records and the float4 from one copy to the next
    uint32_t tri_stride;
    const float4* insts; // instance records; nullptr for single-level scenes
    uint32_t mask;       // instance mask of the ray
    float3 o, d, inv;    // the ray in the current space (object space inside an instance)
    float tmin;
    RayPre pre;
    uint2 ngroup, tgroup;
    Hit best;          // a hit was found once best.geom != kNoInst
    float det;         // GBPT_DEFER_UV: best.u, best.v are V, W of the test until divided by it
    float3 wo, wd; // the world ray
    uint32_t inst; // instance being traversed, kNoInst at the top level
    int inst_sp;   // stack depth at which it was entered
    // the traversal stack's depth, kept in bits 24..31 of the ray's axis word
    GBPT_DI int sp() const { return (int)(pre.k >> 24); }
    GBPT_DI void push_sp() { pre.k += 1u << 24; }
    GBPT_DI void pop_sp() { pre.k -= 1u << 24; }
    GBPT_DI void clear_sp() { pre.k &= 0x00FFFFFFu; }
};

GBPT_DI void set_ray(TraceState& s, float3 o, float3 d) {
    s.o = o;
    s.d = d;
    s.inv = f3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
    const uint32_t oct = (__float_as_uint(d.x) >> 31) | ((__float_as_uint(d.y) >> 31) << 1) |
                         ((__float_as_uint(d.z) >> 31) << 2);
    const uint32_t depth = s.pre.k & 0xFF000000u; // the stack outlives a change of space
    s.pre = ray_pre(o, d);
    s.pre.k |= ((7u - oct) << 8) | ((s.mask & 0xFFu) << 16) | depth;
    s.tris = kTriCopies > 1 ? s.tris_base + (size_t)s.pre.kz() * s.tri_stride : s.tris_base;
}

GBPT_DI void trace_init(TraceState& s, float3 o, float3 d, float tmin, float tmax) {
    s.pre.k = 0u;
    set_ray(s, o, d);
    s.wo = o;
    s.wd = d;
    s.tmin = tmin;
    s.ngroup = make_uint2(0u, 0x80000000u);
    s.tgroup = make_uint2(0u, 0u);
    s.best.t = tmax;
    s.best.u = s.best.v = 0.0f;
    s.best.prim = s.best.geom = s.best.inst = kNoInst;
    s.inst = kNoInst;
    s.inst_sp = -1;
}

GBPT_DI void enter_instance(TraceState& s, uint32_t ii) {
    const float4* r = s.insts + 7ull * ii;
    const float4 w0 = __ldg(r + 3), w1 = __ldg(r + 4), w2 = __ldg(r + 5);
    set_ray(s, xform_point(w0, w1, w2, s.wo), xform_vector(w0, w1, w2, s.wd));
    s.inst = ii;
    s.inst_sp = s.sp();
    s.ngroup = make_uint2(__float_as_uint(__ldg(r + 6).x), 0x80000000u);
}

GBPT_DI void exit_instance(TraceState& s) {
    set_ray(s, s.wo, s.wd);
    s.inst = kNoInst;
    s.inst_sp = -1;
}

// Child box planes. Byte j of a plane word w is the quantised plane q of child j; the slab
// distance is t = q * a + o, a = 2^e / d and o = (p - origin) / d per node and axis.
// GBPT_BOX_BIAS (the default): one byte permute writes q into bits 8..15 of the float 32768.0,
// which makes the float 32768 + q exactly, and the per-node offsets absorb the bias
// (o' = o - 32768 a), so a plane costs a permute and an FMA. The rounding of o' is at most
// 2^-9 |a| (a 512th of a quantisation step); the slack below covers it. Without it: shift, mask
// and integer-to-float conversion, then the FMA.
#ifndef GBPT_BOX_BIAS
#define GBPT_BOX_BIAS 1
#endif
#if GBPT_BOX_BIAS
constexpr float kPlaneBias = 32768.0f;
GBPT_DI float qplane(uint32_t w, int j) {
    return __uint_as_float(__byte_perm(w, 0x47000000u, 0x7504u | ((uint32_t)j << 4)));
}
#else
constexpr float kPlaneBias = 0.0f;
GBPT_DI float qplane(uint32_t w, int j) { return (float)((w >> (8 * j)) & 0xFFu); }
#endif

// GBPT_BOX_FMA2: the plane distances of two children with one paired FP32 FMA (fma.rn.f32x2).
#ifndef GBPT_BOX_FMA2
#define GBPT_BOX_FMA2 1
#endif
GBPT_DI uint64_t pack2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
// the biased planes of children J and J + 1 of word w (as qplane), times a plus o, per lane
template <int J> GBPT_DI float2 plane_t2(uint32_t w, uint64_t a2, uint64_t o2) {
    float2 r;
    asm("{\n\t.reg .b32 q0, q1;\n\t.reg .b64 q, d;\n\t"
        "prmt.b32 q0, %2, 0x47000000, %3;\n\t"
        "prmt.b32 q1, %2, 0x47000000, %4;\n\t"
        "mov.b64 q, {q0, q1};\n\t"
        "fma.rn.f32x2 d, q, %5, %6;\n\t"
        "mov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "r"(w), "n"(0x7504 | (J << 4)), "n"(0x7504 | ((J + 1) << 4)), "l"(a2), "l"(o2));
    return r;
}

// Intersects the 8 children of node `ni`; returns the hit mask (inner children in bits 24..31 in
// traversal order, triangles in bits 0..23) and the node's child / triangle bases and imask.
// The quantised planes are dequantised with a per-axis slack of 2^-20 of the plane distance
// magnitude (plus 2^-8 of a quantisation step for the biased planes), so rounding never loses a
// child the exact box would keep.
template <bool COUNT, bool PAIRED = GBPT_BOX_FMA2 != 0>
GBPT_DI uint32_t intersect_node(const TraceState& s, uint32_t ni, uint32_t& child_base,
                                uint32_t& tri_base, uint32_t& imask, TraceCounters* ctr) {
    if (COUNT) ctr->nodes++;
    const uint4 n0 = __ldg(&s.nodes[5 * ni + 0]);
    const uint4 n1 = __ldg(&s.nodes[5 * ni + 1]);
    const uint4 n2 = __ldg(&s.nodes[5 * ni + 2]);
    const uint4 n3 = __ldg(&s.nodes[5 * ni + 3]);
    const uint4 n4 = __ldg(&s.nodes[5 * ni + 4]);
    const float kErr = 1.0f / 1048576.0f;
    const float kBiasErr = GBPT_BOX_BIAS ? 1.0f / 256.0f : 0.0f;
    // every operation rounded once in a fixed order (no contraction choices left to the
    // compiler), so a host walk of the same tree makes the same box decisions
    const float aix = __fmul_rn(__uint_as_float((n0.w & 0xFFu) << 23), s.inv.x);
    const float aiy = __fmul_rn(__uint_as_float(((n0.w >> 8) & 0xFFu) << 23), s.inv.y);
    const float aiz = __fmul_rn(__uint_as_float(((n0.w >> 16) & 0xFFu) << 23), s.inv.z);
    const float aox = __fmul_rn(__fsub_rn(__uint_as_float(n0.x), s.o.x), s.inv.x);
    const float aoy = __fmul_rn(__fsub_rn(__uint_as_float(n0.y), s.o.y), s.inv.y);
    const float aoz = __fmul_rn(__fsub_rn(__uint_as_float(n0.z), s.o.z), s.inv.z);
    const float ex = __fmaf_rn(kBiasErr, fabsf(aix),
                               __fmul_rn(__fmaf_rn(255.0f, fabsf(aix), fabsf(aox)), kErr));
    const float ey = __fmaf_rn(kBiasErr, fabsf(aiy),
                               __fmul_rn(__fmaf_rn(255.0f, fabsf(aiy), fabsf(aoy)), kErr));
    const float ez = __fmaf_rn(kBiasErr, fabsf(aiz),
                               __fmul_rn(__fmaf_rn(255.0f, fabsf(aiz), fabsf(aoz)), kErr));
    const float nox = __fmaf_rn(-kPlaneBias, aix, __fsub_rn(aox, ex));
    const float fox = __fmaf_rn(-kPlaneBias, aix, __fadd_rn(aox, ex));
    const float noy = __fmaf_rn(-kPlaneBias, aiy, __fsub_rn(aoy, ey));
    const float foy = __fmaf_rn(-kPlaneBias, aiy, __fadd_rn(aoy, ey));
    const float noz = __fmaf_rn(-kPlaneBias, aiz, __fsub_rn(aoz, ez));
    const float foz = __fmaf_rn(-kPlaneBias, aiz, __fadd_rn(aoz, ez));
    imask = n0.w >> 24;
    child_base = n1.x;
    tri_base = n1.y;

    // the direction's signs from the octant (negative axis a: bit a of oct_inv clear)
    const uint32_t oct_inv = s.pre.oct_inv();
    const uint32_t oct_inv4 = oct_inv * 0x01010101u;
    const bool negx = (oct_inv & 1u) == 0u, negy = (oct_inv & 2u) == 0u;
    const bool negz = (oct_inv & 4u) == 0u;
    uint32_t hitmask = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const uint32_t meta4 = half ? n1.w : n1.z;
        const uint32_t is_inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
        const uint32_t inner_mask4 = (is_inner4 >> 4) * 0xFFu;
        const uint32_t bit_index4 = (meta4 ^ (oct_inv4 & inner_mask4)) & 0x1F1F1F1Fu;
        const uint32_t child_bits4 = (meta4 >> 5) & 0x07070707u;
        const uint32_t qlx = half ? n2.y : n2.x, qly = half ? n2.w : n2.z;
        const uint32_t qlz = half ? n3.y : n3.x, qhx = half ? n3.w : n3.z;
        const uint32_t qhy = half ? n4.y : n4.x, qhz = half ? n4.w : n4.z;
        const uint32_t nqx = negx ? qhx : qlx, fqx = negx ? qlx : qhx;
        const uint32_t nqy = negy ? qhy : qly, fqy = negy ? qly : qhy;
        const uint32_t nqz = negz ? qhz : qlz, fqz = negz ? qlz : qhz;
        if constexpr (PAIRED) {
            // children j and j + 1 of the half at once: the paired FP32 FMA rounds each lane like
            // __fmaf_rn, so the decisions are the scalar ones
            const uint64_t ax2 = pack2(aix, aix), ay2 = pack2(aiy, aiy), az2 = pack2(aiz, aiz);
            const uint64_t nox2 = pack2(nox, nox), noy2 = pack2(noy, noy), noz2 = pack2(noz, noz);
            const uint64_t fox2 = pack2(fox, fox), foy2 = pack2(foy, foy), foz2 = pack2(foz, foz);
            auto pair = [&](auto jc) {
                constexpr int j = decltype(jc)::value;
                const float2 tnx = plane_t2<j>(nqx, ax2, nox2), tny = plane_t2<j>(nqy, ay2, noy2);
                const float2 tnz = plane_t2<j>(nqz, az2, noz2), tfx = plane_t2<j>(fqx, ax2, fox2);
                const float2 tfy = plane_t2<j>(fqy, ay2, foy2), tfz = plane_t2<j>(fqz, az2, foz2);
                const float cmin0 = fmaxf(fmaxf(tnx.x, tny.x), fmaxf(tnz.x, s.tmin));
                const float cmax0 = fminf(fminf(tfx.x, tfy.x), fminf(tfz.x, s.best.t));
                const float cmin1 = fmaxf(fmaxf(tnx.y, tny.y), fmaxf(tnz.y, s.tmin));
                const float cmax1 = fminf(fminf(tfx.y, tfy.y), fminf(tfz.y, s.best.t));
                constexpr uint32_t sh0 = 8u * j, sh1 = 8u * (j + 1);
                if (cmin0 <= cmax0)
                    hitmask |= ((child_bits4 >> sh0) & 7u) << ((bit_index4 >> sh0) & 31u);
                if (cmin1 <= cmax1)
                    hitmask |= ((child_bits4 >> sh1) & 7u) << ((bit_index4 >> sh1) & 31u);
            };
            pair(std::integral_constant<int, 0>{});
            pair(std::integral_constant<int, 2>{});
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t sh = 8u * j;
                const float tnx = __fmaf_rn(qplane(nqx, j), aix, nox);
                const float tny = __fmaf_rn(qplane(nqy, j), aiy, noy);
                const float tnz = __fmaf_rn(qplane(nqz, j), aiz, noz);
                const float tfx = __fmaf_rn(qplane(fqx, j), aix, fox);
                const float tfy = __fmaf_rn(qplane(fqy, j), aiy, foy);
                const float tfz = __fmaf_rn(qplane(fqz, j), aiz, foz);
                const float cmin = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, s.tmin));
                const float cmax = fminf(fminf(tfx, tfy), fminf(tfz, s.best.t));
                if (cmin <= cmax)
                    hitmask |= ((child_bits4 >> sh) & 7u) << ((bit_index4 >> sh) & 31u);
            }
        }
    }
    return hitmask;
}

// Runs the traversal of the ray in s until it is finished (returns true; result in s.best, geom
// = kNoInst on a miss; with ANY the first hit found) or, with WARP, until the warp should refill
// its idle lanes (returns false; s keeps the state). `st(i)` is stack entry i. A stack overflow
// raises *err and finishes the ray with what it found.
// `alpha(geom, prim, u, v)` decides the candidate hits of non-opaque triangles (true: skip).
template <bool ANY, bool COUNT, bool TWO_LEVEL, bool WARP, class StackRef, class Alpha>
GBPT_DI bool trace_loop(TraceState& s, StackRef&& st, TraceCounters* ctr, uint32_t* err,
                        bool pool_empty, const Alpha& alpha, int refill_lanes = 0,
                        int postpone_lanes = 0) {
    while (true) {
        if (s.ngroup.y > 0x00FFFFFFu) {
            const uint32_t hits = s.ngroup.y;
            const uint32_t bit = 31u - __clz(hits & 0xFF000000u);
            s.ngroup.y &= ~(1u << bit);
            if (s.ngroup.y > 0x00FFFFFFu) {
                if (s.sp() >= kStackSize) {
                    atomicOr(err, 1u);
                    s.clear_sp();
                    s.ngroup.y = 0;
                    s.tgroup.y = 0;
                    s.inst = kNoInst;
                    break;
                }
                st(s.sp()) = s.ngroup;
                s.push_sp();
            }
            const uint32_t slot = (bit - 24u) ^ s.pre.oct_inv();
            const uint32_t ni = s.ngroup.x + __popc((hits & 0xFFu) & ((1u << slot) - 1u));
            uint32_t cb, tb, im;
            if (COUNT) count_step(ctr->node_steps, ctr->node_lanes);
            // the paired planes hold more registers: first-hit traversal, which keeps fewer,
            // measured faster with the scalar ones
            const uint32_t hm =
                intersect_node<COUNT, GBPT_BOX_FMA2 != 0 && !ANY>(s, ni, cb, tb, im, ctr);
            s.ngroup = make_uint2(cb, (hm & 0xFF000000u) | im);
            s.tgroup = make_uint2(tb, hm & 0x00FFFFFFu);
        } else {
            // a postponed triangle group (or the rest of a top-level instance group) came off
            // the stack
            s.tgroup = s.ngroup;
            s.ngroup = make_uint2(0u, 0u);
        }
        bool done_any = false;
        // only groups followed by node work are postponed (a group popped back is tested), and
        // never those of a first-hit query, which any of its triangles may end
        const bool may_postpone = WARP && !ANY && s.ngroup.y > 0x00FFFFFFu;
        while (s.tgroup.y != 0u) {
            if (may_postpone && s.sp() < kStackSize && __popc(__activemask()) < postpone_lanes) {
                st(s.sp()) = s.tgroup;
                s.push_sp();
                s.tgroup.y = 0u;
                break;
            }
            const uint32_t b = __ffs(s.tgroup.y) - 1u;
            s.tgroup.y &= s.tgroup.y - 1u;
            const uint32_t ti = s.tgroup.x + b;
            if (TWO_LEVEL && s.insts != nullptr && s.inst == kNoInst) {
                // a top-level leaf: an instance (record: instance index, mask in the flag word)
                const uint32_t fl = __float_as_uint(__ldg(&s.tris[3 * ti + 2]).w);
                if ((fl & s.pre.mask()) == 0u) continue;
                if (s.sp() + 2 > kStackSize) {
                    atomicOr(err, 1u);
                    s.tgroup.y = 0u;
                    continue;
                }
                if (s.ngroup.y > 0x00FFFFFFu) {
                    st(s.sp()) = s.ngroup;
                    s.push_sp();
                }
                if (s.tgroup.y != 0u) {
                    st(s.sp()) = s.tgroup;
                    s.push_sp();
                }
                s.tgroup.y = 0u;
                enter_instance(s, __float_as_uint(__ldg(&s.tris[3 * ti]).w));
                break;
            }
            const float4* rec = s.tris + 3 * ti;
            const float4 r0 = __ldg(rec + 0);
            const float4 r1 = __ldg(rec + 1);
            const float4 r2 = __ldg(rec + 2);
            const uint32_t tfl = __float_as_uint(r2.w);
            if ((tfl & s.pre.mask()) == 0u) continue;
            if (COUNT) {
                ctr->tris++;
                count_step(ctr->tri_steps, ctr->tri_lanes);
            }
            float t, u, v;
            float det;
            if (!intersect_tri(s.pre, r0, r1, r2, tfl, s.tmin, s.best.t, t, u, v, det)) continue;
            const uint32_t prim = __float_as_uint(r0.w), geom = __float_as_uint(r1.w);
            if (t < s.best.t || geom < s.best.geom ||
                (geom == s.best.geom &&
                 (prim < s.best.prim || (prim == s.best.prim && s.inst < s.best.inst)))) {
#if GBPT_DEFER_UV
                if ((tfl & kTriAlpha) && alpha(geom, prim, __fdiv_rn(u, det), __fdiv_rn(v, det)))
                    continue;
                s.det = det;
#else
                if ((tfl & kTriAlpha) && alpha(geom, prim, u, v)) continue;
#endif
                s.best.t = t;
                s.best.u = u;
                s.best.v = v;
                s.best.prim = prim;
                s.best.geom = geom;
                s.best.inst = s.inst;
                if (ANY) {
                    done_any = true;
                    break;
                }
            }
        }
        bool done = done_any;
        if (!done && s.ngroup.y <= 0x00FFFFFFu) {
            if (TWO_LEVEL && s.inst != kNoInst && s.sp() == s.inst_sp) exit_instance(s);
            if (s.sp() == 0) {
                done = true;
            } else {
                s.pop_sp();
                s.ngroup = st(s.sp());
            }
        }
        if (done) break;
        if (WARP && !pool_empty && __popc(__activemask()) < refill_lanes) return false;
    }
#if GBPT_DEFER_UV
    if (s.best.geom != kNoInst) {
        s.best.u = __fdiv_rn(s.best.u, s.det);
        s.best.v = __fdiv_rn(s.best.v, s.det);
    }
#endif
    return true;
}

// Closest hit (ANY = false) or first hit (ANY = true) of one ray, per thread. Sets *err when the
// traversal stack would overflow (the builder bounds the depth, so this does not happen for
// trees it accepted).
template <bool ANY, bool COUNT>
__device__ __forceinline__ Hit trace_ray(const DevScene& sc, float3 o, float3 d, float tmin,
                                         float tmax, uint32_t ray_mask, TraceCounters* ctr,
                                         uint32_t* err) {
    TraceState s;
    s.nodes = sc.nodes;
    s.tris_base = sc.tris;
    s.tri_stride = sc.tri_stride;
    s.insts = sc.n_inst ? sc.inst : nullptr;
    s.mask = ray_mask;
    trace_init(s, o, d, tmin, tmax);
    uint2 stack[kStackSize];
    trace_loop<ANY, COUNT, true, false>(
        s, [&](int i) -> uint2& { return stack[i]; }, ctr, err, true,
        [&](uint32_t g, uint32_t p, float u, float v) { return alpha_discard(sc, g, p, u, v); });
    return s.best;
}

// Runs the traversal of every ray i < n with persistent warps that pull ray indices from *fetch
// (zero before the launch; one atomic per warp for all idle lanes). load(i, state) sets ray i's
// scene (nodes, tris, insts), mask and calls trace_init; store(i, hit) receives its result;
// alpha(i, geom, prim, u, v) is ray i's alpha test (true: skip the candidate). Must be called by
// all 32 lanes of every warp.
template <bool ANY, bool COUNT, bool TWO_LEVEL, class Load, class Store, class Alpha>
__device__ __forceinline__ void trace_persistent(uint32_t n, uint32_t* fetch, Load load,
                                                 Store store, Alpha alpha, TraceCounters* ctr,
                                                 uint32_t* err, int refill_lanes,
                                                 int postpone_lanes) {
    const uint32_t lane = threadIdx.x & 31u;
    uint2 stack[kStackSize];
    auto st_ref = [&](int i) -> uint2& { return stack[i]; };
    TraceState s;
    uint32_t ray = 0xFFFFFFFFu;
    bool active = false, exhausted = false;
    while (true) {
        __syncwarp();
        const bool want = !active && !exhausted;
        const uint32_t want_mask = __ballot_sync(0xFFFFFFFFu, want);
        if (want_mask) {
            const uint32_t leader = __ffs(want_mask) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(want_mask));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (want) {
                ray = base + __popc(want_mask & ((1u << lane) - 1u));
                if (ray < n) {
                    load(ray, s);
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, active) == 0u) break;
        // once a lane found the pool empty, leaving the loop to refill gains nothing
        const bool pool_empty = __ballot_sync(0xFFFFFFFFu, exhausted) != 0u;
        if (!active) continue;
        const auto ray_alpha = [&](uint32_t g, uint32_t p, float u, float v) {
            return alpha(ray, g, p, u, v);
        };
        if (trace_loop<ANY, COUNT, TWO_LEVEL, true>(s, st_ref, ctr, err, pool_empty, ray_alpha,
                                                    refill_lanes, postpone_lanes)) {
            store(ray, s.best);
            active = false;
        }
    }
}

// ---- camera (camera.slang:29-56), bit-identical to the oracle's FP32 build ---------------------------
struct CamGPU {
    float3 pos, U, V, W;
    float near_plane, far_plane, jx, jy;
};
GBPT_DI void camera_ray(const CamGPU& c, uint32_t px, uint32_t py, uint32_t w, uint32_t h,
                        float3& o, float3& d, float& tmin, float& tmax) {
    const float x = __fdiv_rn(__fadd_rn(__fadd_rn((float)px, 0.5f), c.jx), (float)w);
    const float y = __fdiv_rn(__fadd_rn(__fadd_rn((float)py, 0.5f), c.jy), (float)h);
    const float nx = __fadd_rn(__fmul_rn(2.0f, x), -1.0f);
    const float ny = __fadd_rn(__fmul_rn(-2.0f, y), 1.0f);
    const float dx = __fadd_rn(__fadd_rn(__fmul_rn(nx, c.U.x), __fmul_rn(ny, c.V.x)), c.W.x);
    const float dy = __fadd_rn(__fadd_rn(__fmul_rn(nx, c.U.y), __fmul_rn(ny, c.V.y)), c.W.y);
    const float dz = __fadd_rn(__fadd_rn(__fmul_rn(nx, c.U.z), __fmul_rn(ny, c.V.z)), c.W.z);
    const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    d = f3(__fdiv_rn(dx, l), __fdiv_rn(dy, l), __fdiv_rn(dz, l));
    const float lw = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.W.x, c.W.x), __fmul_rn(c.W.y, c.W.y)),
                                          __fmul_rn(c.W.z, c.W.z)));
    const float wx = __fdiv_rn(c.W.x, lw), wy = __fdiv_rn(c.W.y, lw), wz = __fdiv_rn(c.W.z, lw);
    const float cosv = __fadd_rn(__fadd_rn(__fmul_rn(wx, d.x), __fmul_rn(wy, d.y)), __fmul_rn(wz, d.z));
    const float inv_cos = __fdiv_rn(1.0f, cosv);
    o = c.pos;
    tmin = __fmul_rn(c.near_plane, inv_cos);
    tmax = __fmul_rn(c.far_plane, inv_cos);
}

// ---- environment (environment-map.slang:23-35, utils/math.slang:243-250) -------------------------------
GBPT_DI float3 env_to_local(const DevScene& s, float3 d) {
    const float* M = s.env_m;
    return f3(M[0] * d.x + M[1] * d.y + M[2] * d.z, M[3] * d.x + M[4] * d.y + M[5] * d.z,
              M[6] * d.x + M[7] * d.y + M[8] * d.z);
}
GBPT_DI int wrapi(int i, int n) {
    const int r = i % n;
    return r < 0 ? r + n : r;
}
// The lat-long map coordinates (u, v) of a world direction (its local frame by env_to_local).
GBPT_DI void env_uv(const DevScene& s, float3 dir, float& u, float& v) {
    const float3 p = normalize(env_to_local(s, dir));
    u = atan2f(p.x, -p.z) * kInv2Pi + 0.5f;
    v = acosf(fminf(fmaxf(p.y, -1.0f), 1.0f)) * kInvPi;
}
// The environment's radiance at map coordinates (u, v): bilinear, repeating.
GBPT_DI float3 env_eval_uv(const DevScene& s, float u, float v) {
    if (!(u == u) || !(v == v)) return f3(0.f, 0.f, 0.f);
    const float x = u * (float)s.ew - 0.5f, y = v * (float)s.eh - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    const int ix = (int)fx, iy = (int)fy;
    const int x0 = wrapi(ix, (int)s.ew), x1 = wrapi(ix + 1, (int)s.ew);
    const int y0 = wrapi(iy, (int)s.eh), y1 = wrapi(iy + 1, (int)s.eh);
    const float4 t00 = __ldg(&s.env[(size_t)y0 * s.ew + x0]);
    const float4 t10 = __ldg(&s.env[(size_t)y0 * s.ew + x1]);
    const float4 t01 = __ldg(&s.env[(size_t)y1 * s.ew + x0]);
    const float4 t11 = __ldg(&s.env[(size_t)y1 * s.ew + x1]);
    const float3 top = f3(t00.x, t00.y, t00.z) * (1.0f - a) + f3(t10.x, t10.y, t10.z) * a;
    const float3 bot = f3(t01.x, t01.y, t01.z) * (1.0f - a) + f3(t11.x, t11.y, t11.z) * a;
    return (top * (1.0f - b) + bot * b) * s.env_intensity;
}
GBPT_DI float3 env_eval(const DevScene& s, float3 dir) {
    if (s.ew == 0u) return f3(0.f, 0.f, 0.f);
    float u, v;
    env_uv(s, dir, u, v);
    return env_eval_uv(s, u, v);
}

} // namespace gbpt

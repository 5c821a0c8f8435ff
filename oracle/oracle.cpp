// ORACLE (test infrastructure only; the product never links or calls this file). CPU restatement
// of merian's `pt` renderer (include/merian-graph/nodes/render_pt/render_pt.slang:24-130) and of
// the scene functions it calls (include/merian-shaders/scene/scene.slang:62-102,312-498,
// hit.slang:7-147), templated on float (the timed CPU baseline) and double (the parity
// estimator). Hardware ray queries have no source in the reference; they are restated as a
// binary binned-SAH BVH with the watertight ray/triangle test of Woop, Benthin and Wald (JCGT
// 2013), back-face culling per merian's MeshFlags (scene.cpp:1841-1848) and a deterministic tie
// rule (smallest geometry, then primitive id, at equal t). Also restates the BSDF property checks
// of tests/bsdf/bsdf-checks.slang and the next-event-estimation estimator that the GPU adds
// (not in the reference; unbiased against it).
#include "oracle_math.h"
#include "host_common.h" // the package's alias-table builder (oracle_alias_table)

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API extern "C" __attribute__((visibility("default")))

namespace oracle {

constexpr uint32_t kNoInst = 0xFFFFFFFFu;

// Triangles and their binary BVH: a whole single-level scene, or one BLAS in object space.
struct TriSet {
    std::vector<float> tv;        // 9 per triangle
    std::vector<uint32_t> tgeom;  // geometry of each triangle
    std::vector<uint32_t> tprim;  // primitive id within the geometry
    struct Node {
        float lo[3], hi[3];
        uint32_t left_or_first, count; // count > 0: leaf over perm[first, first+count)
    };
    std::vector<Node> nodes;
    std::vector<uint32_t> perm;
};

// A TLAS instance: row-major 3x4 transforms (world-to-object computed in double, rounded once,
// exactly as the library computes it), BLAS, mask, first geometry and world bounds.
struct Instance {
    float o2w[12], w2o[12];
    uint32_t blas, mask, first_geom;
    double lo[3], hi[3];
};

struct Scene : TriSet {
    std::vector<gbpt_packed_vertex> verts;
    std::vector<uint32_t> idx;
    std::vector<gbpt_geometry> geoms;
    std::vector<gbpt_material> mats;
    std::vector<float> env;
    uint32_t ew = 0, eh = 0;
    float env_to_local[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    float env_intensity = 1.0f;
    // the flattened triangles (TriSet, in the order of `idx`) of a single-level scene
    std::vector<uint32_t> geom_tri_base; // first flattened triangle of each geometry
    // two-level scenes
    std::vector<TriSet> blas;
    std::vector<Instance> insts;
    // RGBA8 textures: texels, (first texel, width, height, sRGB) per texture, sRGB decode table
    std::vector<uint8_t> tex;
    std::vector<uint32_t> tex_info;
    float srgb_lut[256] = {};
    // emissive triangles for next-event estimation, in world space (one copy per instance)
    std::vector<float> light_tv;       // 9 per light
    std::vector<uint32_t> light_geom;
    std::vector<uint32_t> light_tri;   // light index (kept for the selection count)
    std::vector<double> light_cdf; // inclusive prefix of power, normalised to 1
    double light_total = 0.0;
    // environment importance sampling
    std::vector<double> env_marg;  // eh + 1, prefix of row sums
    std::vector<double> env_cond;  // eh * (ew + 1) per-row prefix
    std::vector<double> env_func;  // eh * ew
    double env_func_int = 0.0;     // sum / (ew*eh)
};

// ---- BVH2 build (binned SAH, 16 bins) ---------------------------------------------------------
static void build_bvh(TriSet& s) {
    const size_t n = s.tgeom.size();
    s.perm.resize(n);
    for (size_t i = 0; i < n; ++i) s.perm[i] = (uint32_t)i;
    std::vector<float> blo(3 * n), bhi(3 * n), cen(3 * n);
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            const float x = s.tv[9 * i + a], y = s.tv[9 * i + 3 + a], z = s.tv[9 * i + 6 + a];
            blo[3 * i + a] = std::min(x, std::min(y, z));
            bhi[3 * i + a] = std::max(x, std::max(y, z));
            cen[3 * i + a] = 0.5f * (blo[3 * i + a] + bhi[3 * i + a]);
        }
    s.nodes.clear();
    s.nodes.push_back({});
    struct T {
        uint32_t node, b, e;
    };
    std::vector<T> st{{0, 0, (uint32_t)n}};
    auto area = [](const float* lo, const float* hi) {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    };
    while (!st.empty()) {
        const T t = st.back();
        st.pop_back();
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = t.b; i < t.e; ++i) {
            const uint32_t p = s.perm[i];
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], blo[3 * p + a]);
                hi[a] = std::max(hi[a], bhi[3 * p + a]);
                clo[a] = std::min(clo[a], cen[3 * p + a]);
                chi[a] = std::max(chi[a], cen[3 * p + a]);
            }
        }
        Scene::Node& nd = s.nodes[t.node];
        std::memcpy(nd.lo, lo, 12);
        std::memcpy(nd.hi, hi, 12);
        const uint32_t cnt = t.e - t.b;
        nd.left_or_first = t.b;
        nd.count = cnt;
        if (cnt <= 2) continue;
        constexpr int NB = 16;
        float best = FLT_MAX;
        int best_axis = -1, best_bin = 0;
        for (int a = 0; a < 3; ++a) {
            const float ext = chi[a] - clo[a];
            if (!(ext > 0.0f)) continue;
            float bl[NB][3], bh[NB][3];
            uint32_t bn[NB] = {};
            for (int b = 0; b < NB; ++b)
                for (int k = 0; k < 3; ++k) bl[b][k] = FLT_MAX, bh[b][k] = -FLT_MAX;
            for (uint32_t i = t.b; i < t.e; ++i) {
                const uint32_t p = s.perm[i];
                int b = (int)((cen[3 * p + a] - clo[a]) / ext * NB);
                b = std::min(std::max(b, 0), NB - 1);
                bn[b]++;
                for (int k = 0; k < 3; ++k) {
                    bl[b][k] = std::min(bl[b][k], blo[3 * p + k]);
                    bh[b][k] = std::max(bh[b][k], bhi[3 * p + k]);
                }
            }
            for (int split = 1; split < NB; ++split) {
                float l0[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, l1[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                float r0[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, r1[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                uint32_t nl = 0, nr = 0;
                for (int b = 0; b < NB; ++b) {
                    float* x0 = b < split ? l0 : r0;
                    float* x1 = b < split ? l1 : r1;
                    (b < split ? nl : nr) += bn[b];
                    for (int k = 0; k < 3; ++k) {
                        x0[k] = std::min(x0[k], bl[b][k]);
                        x1[k] = std::max(x1[k], bh[b][k]);
                    }
                }
                if (nl == 0 || nr == 0) continue;
                const float c = area(l0, l1) * nl + area(r0, r1) * nr;
                if (c < best) {
                    best = c;
                    best_axis = a;
                    best_bin = split;
                }
            }
        }
        uint32_t mid;
        if (best_axis < 0) {
            mid = t.b + cnt / 2;
        } else {
            const float ext = chi[best_axis] - clo[best_axis];
            auto it = std::partition(s.perm.begin() + t.b, s.perm.begin() + t.e, [&](uint32_t p) {
                int b = (int)((cen[3 * p + best_axis] - clo[best_axis]) / ext * NB);
                b = std::min(std::max(b, 0), NB - 1);
                return b < best_bin;
            });
            mid = (uint32_t)(it - s.perm.begin());
            if (mid == t.b || mid == t.e) mid = t.b + cnt / 2;
        }
        const uint32_t l = (uint32_t)s.nodes.size();
        s.nodes.push_back({});
        s.nodes.push_back({});
        s.nodes[t.node].left_or_first = l;
        s.nodes[t.node].count = 0;
        st.push_back({l, t.b, mid});
        st.push_back({l + 1, mid, t.e});
    }
}

// ---- watertight ray/triangle test (Woop, Benthin, Wald 2013) ----------------------------------
// Front face = counter-clockwise (face normal cross(e01, e02) towards the ray origin): U, V, W
// and det all positive. FlipFacing swaps the accepted side, TwoSided accepts both (merian
// MeshFlags, scene.hpp:39-58, mapped to the TLAS instance flags at scene.cpp:1841-1848).
template <class R> struct RayPre {
    int kx, ky, kz;
    bool flip; // direction negative along kz: the 2D frame (kx, ky) sees triangles mirrored
    R Sx, Sy, Sz;
    V3<R> o;
};
template <class R> inline R comp(V3<R> v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
template <class R> inline RayPre<R> ray_pre(const Ray<R>& r) {
    RayPre<R> p;
    const R ax = std::fabs(r.d.x), ay = std::fabs(r.d.y), az = std::fabs(r.d.z);
    p.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    p.kx = (p.kz + 1) % 3;
    p.ky = (p.kx + 1) % 3;
    // the paper swaps kx and ky here to keep the winding; the same frame for both signs negates
    // U, V, W, det and T instead, so t, u and v are unchanged and only the facing flips
    p.flip = comp(r.d, p.kz) < R(0);
    p.Sx = comp(r.d, p.kx) / comp(r.d, p.kz);
    p.Sy = comp(r.d, p.ky) / comp(r.d, p.kz);
    p.Sz = R(1) / comp(r.d, p.kz);
    p.o = r.o;
    return p;
}
struct HitRec {
    double t;
    float u, v;
    uint32_t geom, prim;
    uint32_t inst; // instance of a two-level hit, kNoInst otherwise
    bool valid;
};
// Returns true and the distance / barycentrics when the triangle is hit within [tmin, tmax].
template <class R>
inline bool intersect(const RayPre<R>& p, const float* tv, uint32_t flags, R tmin, R tmax, R& t_out,
                      R& u_out, R& v_out) {
    const V3<R> A = mk<R>(tv[0], tv[1], tv[2]) - p.o;
    const V3<R> B = mk<R>(tv[3], tv[4], tv[5]) - p.o;
    const V3<R> Cc = mk<R>(tv[6], tv[7], tv[8]) - p.o;
    const R Ax = comp(A, p.kx) - p.Sx * comp(A, p.kz);
    const R Ay = comp(A, p.ky) - p.Sy * comp(A, p.kz);
    const R Bx = comp(B, p.kx) - p.Sx * comp(B, p.kz);
    const R By = comp(B, p.ky) - p.Sy * comp(B, p.kz);
    const R Cx = comp(Cc, p.kx) - p.Sx * comp(Cc, p.kz);
    const R Cy = comp(Cc, p.ky) - p.Sy * comp(Cc, p.kz);
    R U = Cx * By - Cy * Bx;
    R V = Ax * Cy - Ay * Cx;
    R W = Bx * Ay - By * Ax;
    if (U == R(0) || V == R(0) || W == R(0)) {
        // edge case: recompute the 2D edge functions in double
        U = (R)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (R)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (R)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < R(0) || V < R(0) || W < R(0)) && (U > R(0) || V > R(0) || W > R(0))) return false;
    const R det = U + V + W;
    if (det == R(0)) return false;
    const bool front = (det > R(0)) != p.flip;
    if (!(flags & GBPT_MESH_TWO_SIDED)) {
        const bool want_front = !(flags & GBPT_MESH_FLIP_FACING);
        if (front != want_front) return false;
    }
    const R Az = p.Sz * comp(A, p.kz);
    const R Bz = p.Sz * comp(B, p.kz);
    const R Cz = p.Sz * comp(Cc, p.kz);
    const R T = U * Az + V * Bz + W * Cz;
    const R t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V / det;
    v_out = W / det;
    return true;
}

// ---- alpha test of non-opaque geometry (material-system.slang:28-38, scene.slang:500-519) -------
// The material's alpha texture, bilinear with repeat addressing at level 0, at the candidate's
// interpolated uv; alpha below 0.5 (merian_alpha_test_threshold) discards the candidate. In the
// FP32 build every operation rounds once in the kernels' order, so decisions match bit for bit.
template <class R> inline R texture_alpha(const Scene& s, uint32_t t, R u, R v) {
    const uint32_t* info = &s.tex_info[4 * t];
    const int w = (int)info[1], h = (int)info[2];
    if (!(std::fabs(u) < R(65536))) u = R(0); // half uvs: only NaN / inf are out of range
    if (!(std::fabs(v) < R(65536))) v = R(0);
    const R x = u * (R)w - R(0.5), y = v * (R)h - R(0.5);
    const R fx = std::floor(x), fy = std::floor(y);
    const R a = x - fx, b = y - fy;
    const int ix = (int)fx, iy = (int)fy;
    auto wrap = [](int i, int n) { return ((i % n) + n) % n; };
    const int x0 = wrap(ix, w), x1 = wrap(ix + 1, w), y0 = wrap(iy, h), y1 = wrap(iy + 1, h);
    auto alpha = [&](int xx, int yy) {
        return (R)s.tex[4 * ((size_t)info[0] + (size_t)yy * w + xx) + 3] * R(1.0f / 255.0f);
    };
    const R ia = R(1) - a, ib = R(1) - b;
    const R top = alpha(x0, y0) * ia + alpha(x1, y0) * a;
    const R bot = alpha(x0, y1) * ia + alpha(x1, y1) * a;
    return top * ib + bot * b;
}

template <class R> inline bool alpha_discard(const Scene& s, uint32_t g, uint32_t prim, R bu, R bv) {
    const gbpt_geometry& geo = s.geoms[g];
    const gbpt_material& m = s.mats[geo.material_id];
    if (m.alpha_texture < 0 || (size_t)m.alpha_texture >= s.tex_info.size() / 4) return false;
    const uint32_t tri = geo.first_triangle + prim;
    R ux[3], uy[3];
    for (int k = 0; k < 3; ++k) {
        const uint32_t uv = s.verts[geo.first_vertex + s.idx[3 * tri + k]].uv;
        ux[k] = (R)half_to_float(uv & 0xffffu);
        uy[k] = (R)half_to_float(uv >> 16);
    }
    const R b0 = (R(1) - bu) - bv;
    const R u = (b0 * ux[0] + bu * ux[1]) + bv * ux[2];
    const R v = (b0 * uy[0] + bu * uy[1]) + bv * uy[2];
    return texture_alpha<R>(s, (uint32_t)m.alpha_texture, u, v) < R(0.5);
}

// Closest (or any) hit of r against one triangle set, updating best / tbest; returns true when an
// any-hit query found its hit. Ties at equal t go to the smallest (geometry, primitive, instance).
template <class R>
static bool trace_set(const Scene& s, const TriSet& ts, const Ray<R>& r, uint32_t mask,
                      bool any_hit, uint32_t inst, HitRec& best, R& tbest, uint64_t* node_count,
                      uint64_t* tri_count) {
    if (ts.nodes.empty() || ts.tgeom.empty()) return false;
    const RayPre<R> pre = ray_pre(r);
    V3<R> inv;
    auto safe_inv = [](R d) {
        const R m = R(1e-20f);
        return R(1) / (std::fabs(d) > m ? d : std::copysign(m, d));
    };
    inv = mk(safe_inv(r.d.x), safe_inv(r.d.y), safe_inv(r.d.z));
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    const R eps = sizeof(R) == 4 ? R(1.0 / (1 << 20)) : R(0);
    while (sp > 0) {
        const uint32_t ni = stack[--sp];
        const TriSet::Node& nd = ts.nodes[ni];
        if (node_count) ++*node_count;
        // slab test, conservative by a relative epsilon in float mode
        R t0 = r.tmin, t1 = tbest;
        bool miss = false;
        for (int a = 0; a < 3 && !miss; ++a) {
            const R o = comp(r.o, a), iv = comp(inv, a);
            R ta = ((R)nd.lo[a] - o) * iv, tb = ((R)nd.hi[a] - o) * iv;
            if (ta > tb) std::swap(ta, tb);
            ta -= std::fabs(ta) * eps;
            tb += std::fabs(tb) * eps;
            t0 = maxr(t0, ta);
            t1 = minr(t1, tb);
            if (t0 > t1) miss = true;
        }
        if (miss) continue;
        if (nd.count > 0) {
            for (uint32_t k = 0; k < nd.count; ++k) {
                const uint32_t tri = ts.perm[nd.left_or_first + k];
                const uint32_t g = ts.tgeom[tri];
                const gbpt_geometry& geo = s.geoms[g];
                if (((geo.instance_mask & 0xFFu) & mask) == 0) continue;
                if (tri_count) ++*tri_count;
                R t, u, v;
                if (!intersect(pre, &ts.tv[9 * tri], geo.flags, r.tmin, tbest, t, u, v)) continue;
                const uint32_t prim = ts.tprim[tri];
                if (!best.valid || t < tbest || g < best.geom ||
                    (g == best.geom && (prim < best.prim || (prim == best.prim && inst < best.inst)))) {
                    if ((geo.flags & GBPT_MESH_ALPHA_TEST) && alpha_discard<R>(s, g, prim, u, v))
                        continue;
                    tbest = t;
                    best.t = (double)t;
                    best.u = (float)u;
                    best.v = (float)v;
                    best.geom = g;
                    best.prim = prim;
                    best.inst = inst;
                    best.valid = true;
                    if (any_hit) return true;
                }
            }
        } else {
            // visit the nearer child first
            const uint32_t l = nd.left_or_first, rr = l + 1;
            const TriSet::Node &a = ts.nodes[l], &b = ts.nodes[rr];
            const int ax = pre.kz;
            const R ca = (R)a.lo[ax] + (R)a.hi[ax], cb = (R)b.lo[ax] + (R)b.hi[ax];
            const bool a_first = (comp(r.d, ax) >= R(0)) ? (ca <= cb) : (ca > cb);
            if (sp + 2 > 128) return false; // depth guard (never reached by the SAH build)
            stack[sp++] = a_first ? rr : l;
            stack[sp++] = a_first ? l : rr;
        }
    }
    return false;
}

// One row of an affine transform applied with one rounding per operation in the order the
// library's kernels use: ((m0 x + m1 y) + m2 z) + m3 w.
template <class R> inline R xform_row(const float* m, V3<R> p, R w) {
    return (((R)m[0] * p.x + (R)m[1] * p.y) + (R)m[2] * p.z) + (R)m[3] * w;
}
template <class R> inline V3<R> xform_point(const float* m, V3<R> p) {
    return mk(xform_row(m, p, R(1)), xform_row(m + 4, p, R(1)), xform_row(m + 8, p, R(1)));
}
template <class R> inline V3<R> xform_vector(const float* m, V3<R> v) {
    return mk(xform_row(m, v, R(0)), xform_row(m + 4, v, R(0)), xform_row(m + 8, v, R(0)));
}

template <class R>
static HitRec trace(const Scene& s, const Ray<R>& r, uint32_t mask, bool any_hit,
                    uint64_t* node_count = nullptr, uint64_t* tri_count = nullptr) {
    HitRec best{};
    best.valid = false;
    best.inst = kNoInst;
    R tbest = r.tmax;
    if (s.insts.empty()) {
        trace_set(s, s, r, mask, any_hit, kNoInst, best, tbest, node_count, tri_count);
        return best;
    }
    // two-level: every instance whose mask and world box the ray meets, in object space (the
    // direction is not renormalised, so t is the world parameter)
    for (uint32_t i = 0; i < (uint32_t)s.insts.size(); ++i) {
        const Instance& in = s.insts[i];
        if ((in.mask & mask) == 0u) continue;
        double t0 = (double)r.tmin, t1 = (double)tbest;
        bool miss = false;
        for (int a = 0; a < 3 && !miss; ++a) {
            const double o = (double)comp(r.o, a), d = (double)comp(r.d, a);
            if (d == 0.0) {
                if (o < in.lo[a] || o > in.hi[a]) miss = true;
                continue;
            }
            double ta = (in.lo[a] - o) / d, tb = (in.hi[a] - o) / d;
            if (ta > tb) std::swap(ta, tb);
            t0 = std::max(t0, ta - 1e-9 * std::fabs(ta));
            t1 = std::min(t1, tb + 1e-9 * std::fabs(tb));
            if (t0 > t1) miss = true;
        }
        if (miss) continue;
        Ray<R> ro;
        ro.o = xform_point<R>(in.w2o, r.o);
        ro.d = xform_vector<R>(in.w2o, r.d);
        ro.tmin = r.tmin;
        ro.tmax = r.tmax;
        if (trace_set(s, s.blas[in.blas], ro, mask, any_hit, i, best, tbest, node_count,
                      tri_count))
            return best;
    }
    return best;
}

// ---- shading point (scene.slang:312-469, hit.slang) ---------------------------------------------
template <class R> struct SP {
    V3<R> pos;
    V3<R> tex_color; // base colour texture at the hit (1 without one)
    uint32_t enc_face_normal;
    V3<R> emission;
    Frame<R> frame;
    bool has_material;
    MaterialBSDF<R> bsdf;
    // for next-event estimation / MIS
    bool emissive_tri;
    bool front;
    uint32_t geom, prim;
};

template <class R> inline V3<R> fetch_pos(const Scene& s, uint32_t vi) {
    const gbpt_packed_vertex& v = s.verts[vi];
    return mk<R>(v.position[0], v.position[1], v.position[2]);
}

// bilinear level-0 sample with repeat addressing of the lat-long map (LatLongMap::eval,
// environment-map.slang:23-35; world_to_latlong_map, utils/math.slang:243-250)
template <class R> V3<R> env_eval(const Scene& s, V3<R> dir) {
    if (s.ew == 0) return mk(R(0), R(0), R(0));
    const float* M = s.env_to_local;
    const V3<R> l = mk<R>((R)M[0] * dir.x + (R)M[1] * dir.y + (R)M[2] * dir.z,
                          (R)M[3] * dir.x + (R)M[4] * dir.y + (R)M[5] * dir.z,
                          (R)M[6] * dir.x + (R)M[7] * dir.y + (R)M[8] * dir.z);
    const V3<R> p = normalize(l);
    const R u = std::atan2(p.x, -p.z) * C<R>::INV_2PI + R(0.5);
    const R v = std::acos(clampr(p.y, R(-1), R(1))) * C<R>::INV_PI;
    if (!(u == u) || !(v == v)) return mk(R(0), R(0), R(0));
    const R x = u * (R)s.ew - R(0.5), y = v * (R)s.eh - R(0.5);
    const R fx = std::floor(x), fy = std::floor(y);
    const R a = x - fx, b = y - fy;
    const long long ix = (long long)fx, iy = (long long)fy;
    auto wrap = [](long long i, long long n) { return (uint32_t)(((i % n) + n) % n); };
    const uint32_t x0 = wrap(ix, s.ew), x1 = wrap(ix + 1, s.ew);
    const uint32_t y0 = wrap(iy, s.eh), y1 = wrap(iy + 1, s.eh);
    auto tex = [&](uint32_t xx, uint32_t yy) {
        const float* t = &s.env[4 * ((size_t)yy * s.ew + xx)];
        return mk<R>(t[0], t[1], t[2]);
    };
    const V3<R> top = tex(x0, y0) * (R(1) - a) + tex(x1, y0) * a;
    const V3<R> bot = tex(x0, y1) * (R(1) - a) + tex(x1, y1) * a;
    return (top * (R(1) - b) + bot * b) * (R)s.env_intensity;
}

template <class R> SP<R> env_sp(const Scene& s, const Ray<R>& ray) {
    SP<R> sp{};
    sp.pos = ray.o + ray.d * R(1e7f); // ENV_MAP_DISTANCE
    sp.enc_face_normal = encode_normal((float)-ray.d.x, (float)-ray.d.y, (float)-ray.d.z);
    sp.emission = env_eval(s, ray.d);
    sp.frame = frame_from_normal(-ray.d);
    sp.has_material = false;
    sp.emissive_tri = false;
    sp.front = true;
    return sp;
}

// get_shading_point(ray, hit) with a valid triangle hit; bary are the Hit barycentrics
// Bilinear lookup with repeat addressing at level 0 (LOD0Sampler, textures.slang:338-423), sRGB
// textures decoded per texel before filtering; returns rgb.
template <class R> inline V3<R> texture_sample(const Scene& s, uint32_t t, R u, R v) {
    const uint32_t* info = &s.tex_info[4 * t];
    const int w = (int)info[1], h = (int)info[2];
    const R x = u * (R)w - R(0.5), y = v * (R)h - R(0.5);
    const R fx = std::floor(x), fy = std::floor(y);
    const R a = x - fx, b = y - fy;
    const int ix = (int)fx, iy = (int)fy;
    auto wrap = [](int i, int n) { return ((i % n) + n) % n; };
    const int x0 = wrap(ix, w), x1 = wrap(ix + 1, w), y0 = wrap(iy, h), y1 = wrap(iy + 1, h);
    auto texel = [&](int xx, int yy) {
        const uint8_t* c = &s.tex[4 * ((size_t)info[0] + (size_t)yy * w + xx)];
        if (info[3]) return mk<R>(s.srgb_lut[c[0]], s.srgb_lut[c[1]], s.srgb_lut[c[2]]);
        return mk<R>((R)c[0] * R(1.0f / 255.0f), (R)c[1] * R(1.0f / 255.0f),
                     (R)c[2] * R(1.0f / 255.0f));
    };
    const V3<R> top = texel(x0, y0) * (R(1) - a) + texel(x1, y0) * a;
    const V3<R> bot = texel(x0, y1) * (R(1) - a) + texel(x1, y1) * a;
    return top * (R(1) - b) + bot * b;
}

// inst: the instance of a two-level hit (position by its object-to-world transform, edges and
// tangents by the linear part, the normal by the inverse transpose; scene.slang:235-259)
template <class R>
SP<R> surface_sp(const Scene& s, const Ray<R>& ray, uint32_t g, uint32_t prim, R bu, R bv, R ior,
                 bool with_material, uint32_t inst = kNoInst) {
    const gbpt_geometry& geo = s.geoms[g];
    if (geo.flags & GBPT_MESH_USE_ENV_MAP) return env_sp(s, ray);
    const uint32_t tri = geo.first_triangle + prim;
    const uint32_t i0 = geo.first_vertex + s.idx[3 * tri + 0];
    const uint32_t i1 = geo.first_vertex + s.idx[3 * tri + 1];
    const uint32_t i2 = geo.first_vertex + s.idx[3 * tri + 2];
    const gbpt_packed_vertex &v0 = s.verts[i0], &v1 = s.verts[i1], &v2 = s.verts[i2];
    const R b0 = R(1) - bu - bv, b1 = bu, b2 = bv;
    const V3<R> p0 = fetch_pos<R>(s, i0), p1 = fetch_pos<R>(s, i1), p2 = fetch_pos<R>(s, i2);
    V3<R> pos = (b0 * p0 + b1 * p1) + b2 * p2;
    V3<R> e01 = p1 - p0, e02 = p2 - p0;
    const float* o2w = inst == kNoInst ? nullptr : s.insts[inst].o2w;
    const float* w2o = inst == kNoInst ? nullptr : s.insts[inst].w2o;
    if (o2w) {
        pos = xform_point<R>(o2w, pos);
        e01 = xform_vector<R>(o2w, e01);
        e02 = xform_vector<R>(o2w, e02);
    }
    V3<R> fn = normalize(cross(e01, e02));
    if (geo.flags & GBPT_MESH_FLIP_FACING) fn = -fn;
    V3<R> vn;
    if (geo.flags & GBPT_MESH_FLAT_SHADING) {
        vn = fn;
    } else {
        vn = normalize((b0 * decode_normal<R>(v0.encoded_normal) +
                        b1 * decode_normal<R>(v1.encoded_normal)) +
                       b2 * decode_normal<R>(v2.encoded_normal));
        if (w2o) // inverse transpose: the columns of the world-to-object rows
            vn = normalize(mk<R>((R)w2o[0] * vn.x + (R)w2o[4] * vn.y + (R)w2o[8] * vn.z,
                                 (R)w2o[1] * vn.x + (R)w2o[5] * vn.y + (R)w2o[9] * vn.z,
                                 (R)w2o[2] * vn.x + (R)w2o[6] * vn.y + (R)w2o[10] * vn.z));
    }
    // tangent: per-vertex, or the UV-derived (Lengyel) fallback
    Frame<R> frame;
    const R uv0x = half_to_float(v0.uv & 0xffffu), uv0y = half_to_float(v0.uv >> 16);
    const R uv1x = half_to_float(v1.uv & 0xffffu), uv1y = half_to_float(v1.uv >> 16);
    const R uv2x = half_to_float(v2.uv & 0xffffu), uv2y = half_to_float(v2.uv >> 16);
    if (geo.flags & GBPT_MESH_HAS_TANGENTS) {
        auto dec_t = [&](uint32_t e, R& w) {
            w = (e & 1u) ? R(-1) : R(1);
            return decode_normal<R>(e & ~1u);
        };
        R w0, w1, w2;
        const V3<R> t0 = dec_t(v0.encoded_tangent, w0), t1 = dec_t(v1.encoded_tangent, w1),
                    t2 = dec_t(v2.encoded_tangent, w2);
        const V3<R> t = (b0 * t0 + b1 * t1) + b2 * t2;
        const R tw = (b0 * w0 + b1 * w1) + b2 * w2;
        V3<R> tn = normalize(t);
        if (o2w) tn = xform_vector<R>(o2w, tn);
        frame = frame_from_tangent(vn, tn, signr(tw));
    } else {
        const R d1x = uv1x - uv0x, d1y = uv1y - uv0y, d2x = uv2x - uv0x, d2y = uv2y - uv0y;
        const R det = d1x * d2y - d2x * d1y;
        if (std::fabs(det) > R(1e-8f)) {
            const R winding = (geo.flags & GBPT_MESH_FLIP_FACING) ? R(1) : R(-1);
            const V3<R> tg = (d2y * e01 - d1y * e02) / det;
            frame = frame_from_tangent(vn, tg, signr(det) * winding);
        } else {
            frame = frame_from_normal(vn);
        }
    }
    V3<R> face_sd = fn;
    bool front = true;
    if (geo.flags & GBPT_MESH_TWO_SIDED) {
        front = dot(-ray.d, fn) >= R(0);
        if (!front) {
            frame.n = -frame.n;
            face_sd = -face_sd;
        }
    }
    (void)face_sd;
    SP<R> sp{};
    sp.pos = pos;
    sp.enc_face_normal = encode_normal((float)fn.x, (float)fn.y, (float)fn.z);
    sp.has_material = with_material;
    sp.geom = g;
    sp.prim = prim;
    const gbpt_material& m = s.mats[geo.material_id];
    const bool emits =
        m.model != GBPT_MATERIAL_DIFFUSE &&
        (m.emission[0] != 0.0f || m.emission[1] != 0.0f || m.emission[2] != 0.0f);
    sp.emission = (emits && front) ? mk<R>(m.emission[0], m.emission[1], m.emission[2])
                                   : mk(R(0), R(0), R(0));
    sp.emissive_tri = emits && front;
    sp.front = front;
    if (m.model == GBPT_MATERIAL_DIFFUSE) {
        // DiffuseMaterial re-orthonormalises through apply_normal_map(0,0,1)
        sp.frame = apply_normal_map(frame, mk(R(0), R(0), R(1)));
    } else {
        sp.frame = frame;
    }
    sp.tex_color = mk(R(1), R(1), R(1));
    if (!s.tex_info.empty() && m.base_color_texture >= 0 &&
        (size_t)m.base_color_texture < s.tex_info.size() / 4) {
        const R u = (b0 * uv0x + b1 * uv1x) + b2 * uv2x;
        const R v = (b0 * uv0y + b1 * uv1y) + b2 * uv2y;
        sp.tex_color = texture_sample<R>(s, (uint32_t)m.base_color_texture, u, v);
    }
    if (with_material) sp.bsdf = make_material<R>(m, sp.tex_color, ior, front);
    return sp;
}

// Hit -> shading point (scene.slang:458-469)
template <class R>
SP<R> shading_point(const Scene& s, const Ray<R>& ray, const HitRec& h, R ior, bool with_material,
                    bool half_bary) {
    if (!h.valid) return env_sp(s, ray);
    R bu = (R)h.u, bv = (R)h.v;
    if (half_bary) { // the GBuffer stores barycentrics as half2 (gbuffer.slang:40-60)
        bu = (R)half_to_float(float_to_half(h.u));
        bv = (R)half_to_float(float_to_half(h.v));
    }
    return surface_sp(s, ray, h.geom, h.prim, bu, bv, ior, with_material, h.inst);
}

// ---- lights for next-event estimation (new in the GB300 build; the reference has none) -------
template <class R> inline R tri_area(const Scene& s, uint32_t tri) {
    const V3<R> a = mk<R>(s.tv[9 * tri], s.tv[9 * tri + 1], s.tv[9 * tri + 2]);
    const V3<R> b = mk<R>(s.tv[9 * tri + 3], s.tv[9 * tri + 4], s.tv[9 * tri + 5]);
    const V3<R> c = mk<R>(s.tv[9 * tri + 6], s.tv[9 * tri + 7], s.tv[9 * tri + 8]);
    return R(0.5) * length(cross(b - a, c - a));
}
static void build_lights(Scene& s) {
    s.light_tri.clear();
    s.light_cdf.clear();
    s.light_tv.clear();
    s.light_geom.clear();
    double acc = 0.0;
    // every placement of an emissive triangle in world space: the flattened triangles of a
    // single-level scene, or each instance's copy of its BLAS triangles
    auto add = [&](const float* tv, uint32_t g, const float* o2w) {
        const gbpt_material& m = s.mats[s.geoms[g].material_id];
        if (m.model == GBPT_MATERIAL_DIFFUSE) return;
        const double lum = 0.299 * m.emission[0] + 0.587 * m.emission[1] + 0.114 * m.emission[2];
        if (!(lum > 0.0)) return;
        float w[9];
        for (int c = 0; c < 3; ++c)
            for (int a = 0; a < 3; ++a) {
                if (!o2w) {
                    w[3 * c + a] = tv[3 * c + a];
                } else {
                    const float* r = o2w + 4 * a;
                    w[3 * c + a] = (float)((double)r[0] * tv[3 * c] + (double)r[1] * tv[3 * c + 1] +
                                           (double)r[2] * tv[3 * c + 2] + (double)r[3]);
                }
            }
        const double e1[3] = {(double)w[3] - w[0], (double)w[4] - w[1], (double)w[5] - w[2]};
        const double e2[3] = {(double)w[6] - w[0], (double)w[7] - w[1], (double)w[8] - w[2]};
        const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                     cz = e1[0] * e2[1] - e1[1] * e2[0];
        const double p = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz) * lum;
        if (!(p > 0.0)) return;
        acc += p;
        s.light_tri.push_back((uint32_t)s.light_geom.size());
        s.light_geom.push_back(g);
        s.light_tv.insert(s.light_tv.end(), w, w + 9);
        s.light_cdf.push_back(acc);
    };
    if (s.insts.empty()) {
        for (uint32_t t = 0; t < s.tgeom.size(); ++t) add(&s.tv[9 * t], s.tgeom[t], nullptr);
    } else {
        for (const Instance& in : s.insts) {
            const TriSet& b = s.blas[in.blas];
            for (uint32_t t = 0; t < b.tgeom.size(); ++t) add(&b.tv[9 * t], b.tgeom[t], in.o2w);
        }
    }
    s.light_total = acc;
    for (double& c : s.light_cdf) c /= acc;
    // environment: piecewise-constant over texels, luminance x sin(theta) with a floor
    s.env_func.clear();
    s.env_marg.clear();
    s.env_cond.clear();
    if (s.ew == 0) return;
    const uint32_t w = s.ew, h = s.eh;
    s.env_func.resize((size_t)w * h);
    double mean = 0.0;
    for (uint32_t y = 0; y < h; ++y) {
        const double st = std::sin(3.14159265358979323846 * (y + 0.5) / h);
        for (uint32_t x = 0; x < w; ++x) {
            const float* t = &s.env[4 * ((size_t)y * w + x)];
            const double l = std::max(0.0, 0.299 * t[0] + 0.587 * t[1] + 0.114 * t[2]);
            s.env_func[(size_t)y * w + x] = l * st;
            mean += l * st;
        }
    }
    mean /= (double)w * h;
    for (double& f : s.env_func) f += 1e-3 * mean + 1e-30;
    s.env_cond.resize((size_t)h * (w + 1));
    s.env_marg.resize(h + 1);
    s.env_marg[0] = 0.0;
    for (uint32_t y = 0; y < h; ++y) {
        double* c = &s.env_cond[(size_t)y * (w + 1)];
        c[0] = 0.0;
        for (uint32_t x = 0; x < w; ++x) c[x + 1] = c[x] + s.env_func[(size_t)y * w + x];
        s.env_marg[y + 1] = s.env_marg[y] + c[w];
    }
    s.env_func_int = s.env_marg[h] / ((double)w * h);
}

} // namespace oracle

// ============================================================================================
// C ABI of the oracle (ctypes from tests, bench's cpu_baseline)
// ============================================================================================
using namespace oracle;

ORACLE_API void* oracle_scene_create(const gbpt_packed_vertex* v, uint64_t nv, const uint32_t* idx,
                                     uint64_t nt, const gbpt_geometry* g, uint32_t ng,
                                     const gbpt_material* m, uint32_t nm, const float* env,
                                     uint32_t ew, uint32_t eh, const float* env_to_local,
                                     float env_intensity) {
    Scene* s = new Scene();
    s->verts.assign(v, v + nv);
    s->idx.assign(idx, idx + 3 * nt);
    s->geoms.assign(g, g + ng);
    s->mats.assign(m, m + nm);
    if (env && ew && eh) {
        s->env.assign(env, env + 4 * (size_t)ew * eh);
        s->ew = ew;
        s->eh = eh;
        if (env_to_local) std::memcpy(s->env_to_local, env_to_local, sizeof(float) * 9);
        s->env_intensity = env_intensity;
    }
    for (uint32_t gi = 0; gi < ng; ++gi) {
        s->geom_tri_base.push_back((uint32_t)s->tgeom.size());
        for (uint32_t k = 0; k < g[gi].triangle_count; ++k) {
            const uint32_t tri = g[gi].first_triangle + k;
            for (int c = 0; c < 3; ++c) {
                const gbpt_packed_vertex& vv = s->verts[g[gi].first_vertex + s->idx[3 * tri + c]];
                for (int a = 0; a < 3; ++a) s->tv.push_back(vv.position[a]);
            }
            s->tgeom.push_back(gi);
            s->tprim.push_back(k);
        }
    }
    build_bvh(*s);
    build_lights(*s);
    return s;
}

ORACLE_API void oracle_scene_destroy(void* s) { delete (Scene*)s; }

// Makes the scene two-level: one BVH per BLAS in object space and the instances (world-to-object
// transforms inverted in double and rounded once, as the library does). Returns -1 on a bad
// range, index or a singular transform.
ORACLE_API int oracle_scene_set_instances(void* sp, const gbpt_blas_range* br, uint32_t nb,
                                          const gbpt_instance* in, uint32_t ni) {
    Scene& s = *(Scene*)sp;
    s.blas.assign(nb, TriSet{});
    for (uint32_t b = 0; b < nb; ++b) {
        if ((uint64_t)br[b].first_geometry + br[b].geometry_count > s.geoms.size()) return -1;
        TriSet& ts = s.blas[b];
        for (uint32_t gi = br[b].first_geometry; gi < br[b].first_geometry + br[b].geometry_count; ++gi) {
            const gbpt_geometry& g = s.geoms[gi];
            for (uint32_t k = 0; k < g.triangle_count; ++k) {
                const uint32_t tri = g.first_triangle + k;
                for (int c = 0; c < 3; ++c) {
                    const gbpt_packed_vertex& vv = s.verts[g.first_vertex + s.idx[3 * tri + c]];
                    for (int a = 0; a < 3; ++a) ts.tv.push_back(vv.position[a]);
                }
                ts.tgeom.push_back(gi);
                ts.tprim.push_back(k);
            }
        }
        build_bvh(ts);
    }
    s.insts.clear();
    for (uint32_t i = 0; i < ni; ++i) {
        Instance x{};
        if (in[i].blas >= nb) return -1;
        std::memcpy(x.o2w, in[i].object_to_world, sizeof(x.o2w));
        const float* m = in[i].object_to_world;
        const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8],
                     h = m[9], k = m[10];
        const double A = e * k - f * h, B = -(d * k - f * g), Cc = d * h - e * g;
        const double det = a * A + b * B + c * Cc;
        if (!(std::fabs(det) > 1e-30)) return -1;
        const double r[9] = {A / det, -(b * k - c * h) / det, (b * f - c * e) / det,
                             B / det, (a * k - c * g) / det,  -(a * f - c * d) / det,
                             Cc / det, -(a * h - b * g) / det, (a * e - b * d) / det};
        const double t[3] = {m[3], m[7], m[11]};
        for (int row = 0; row < 3; ++row) {
            for (int col = 0; col < 3; ++col) x.w2o[4 * row + col] = (float)r[3 * row + col];
            x.w2o[4 * row + 3] = (float)(-(r[3 * row] * t[0] + r[3 * row + 1] * t[1] +
                                           r[3 * row + 2] * t[2]));
        }
        x.blas = in[i].blas;
        x.mask = in[i].mask & 0xFFu;
        x.first_geom = br[in[i].blas].first_geometry;
        for (int q = 0; q < 3; ++q) {
            x.lo[q] = INFINITY;
            x.hi[q] = -INFINITY;
        }
        const TriSet& ts = s.blas[in[i].blas];
        for (size_t v = 0; v < ts.tv.size() / 3; ++v)
            for (int q = 0; q < 3; ++q) {
                const double w = (double)m[4 * q] * ts.tv[3 * v] + (double)m[4 * q + 1] * ts.tv[3 * v + 1] +
                                 (double)m[4 * q + 2] * ts.tv[3 * v + 2] + (double)m[4 * q + 3];
                x.lo[q] = std::min(x.lo[q], w);
                x.hi[q] = std::max(x.hi[q], w);
            }
        for (int q = 0; q < 3; ++q) { // cover the float rounding of transformed positions
            const double pad = 1e-6 * (std::fabs(x.lo[q]) + std::fabs(x.hi[q]) + 1.0);
            x.lo[q] -= pad;
            x.hi[q] += pad;
        }
        s.insts.push_back(x);
    }
    build_lights(s);
    return 0;
}

// RGBA8 textures and the sRGB decoding table (IEC 61966-2-1, in double, rounded once).
ORACLE_API int oracle_scene_set_textures(void* sp, const gbpt_texture* t, uint32_t n) {
    Scene& s = *(Scene*)sp;
    s.tex.clear();
    s.tex_info.clear();
    uint64_t total = 0;
    for (uint32_t i = 0; i < n; ++i) {
        s.tex_info.insert(s.tex_info.end(), {(uint32_t)total, t[i].width, t[i].height,
                                             t[i].srgb ? 1u : 0u});
        s.tex.insert(s.tex.end(), t[i].texels, t[i].texels + 4ull * t[i].width * t[i].height);
        total += (uint64_t)t[i].width * t[i].height;
    }
    for (int i = 0; i < 256; ++i) {
        const double c = i / 255.0;
        s.srgb_lut[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
    return 0;
}

// merian's Hit: for a two-level hit the instance's custom index (the first geometry of its
// BLAS), the TLAS instance and the geometry within the BLAS
template <class R>
static void fill_hit(const Scene& s, const HitRec& h, gbpt_hit& o) {
    if (h.valid) {
        const uint32_t first = h.inst == kNoInst ? 0u : s.insts[h.inst].first_geom;
        o.instance_id = first;
        o.instance_index = h.inst == kNoInst ? 0u : h.inst;
        o.primitive_id = h.prim;
        o.geometry_index = h.geom - first;
        o.barycentrics[0] = h.u;
        o.barycentrics[1] = h.v;
        o.t = (float)h.t;
    } else {
        o.instance_id = o.instance_index = o.primitive_id = o.geometry_index = 0xFFFFFFFFu;
        o.barycentrics[0] = o.barycentrics[1] = 0.0f;
        o.t = -1.0f;
    }
    o.reserved = 0;
}

// Primary hits of a pinhole camera (the GBuffer node's trace, gbuffer_rt.slang:18-27); out_t64
// (optional) receives the distance in the oracle's precision.
ORACLE_API int oracle_trace_primary(void* sp, const gbpt_camera* cam, uint32_t w, uint32_t h,
                                    uint32_t mask, int fp64, gbpt_hit* out, double* out_t64) {
    const Scene& s = *(const Scene*)sp;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)w * h; ++i) {
        const uint32_t px = (uint32_t)(i % w), py = (uint32_t)(i / w);
        HitRec hr;
        if (fp64) {
            hr = trace<double>(s, camera_ray<double>(*cam, px, py, w, h), mask, false);
        } else {
            hr = trace<float>(s, camera_ray<float>(*cam, px, py, w, h), mask, false);
        }
        fill_hit<float>(s, hr, out[i]);
        if (out_t64) out_t64[i] = hr.valid ? hr.t : -1.0;
    }
    return 0;
}

ORACLE_API int oracle_trace_rays(void* sp, const gbpt_ray* rays, uint32_t n, uint32_t mask,
                                 int fp64, int any_hit, gbpt_hit* out, uint64_t* nodes_visited,
                                 uint64_t* tris_tested) {
    const Scene& s = *(const Scene*)sp;
    std::atomic<uint64_t> nn{0}, nt{0};
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        uint64_t a = 0, b = 0;
        HitRec hr;
        if (fp64) {
            Ray<double> r{mk<double>(rays[i].origin[0], rays[i].origin[1], rays[i].origin[2]),
                          mk<double>(rays[i].direction[0], rays[i].direction[1],
                                     rays[i].direction[2]),
                          rays[i].tmin, rays[i].tmax};
            hr = trace<double>(s, r, mask, any_hit != 0, &a, &b);
        } else {
            Ray<float> r{mk<float>(rays[i].origin[0], rays[i].origin[1], rays[i].origin[2]),
                         mk<float>(rays[i].direction[0], rays[i].direction[1],
                                   rays[i].direction[2]),
                         rays[i].tmin, rays[i].tmax};
            hr = trace<float>(s, r, mask, any_hit != 0, &a, &b);
        }
        fill_hit<float>(s, hr, out[i]);
        nn += a;
        nt += b;
    }
    if (nodes_visited) *nodes_visited = nn;
    if (tris_tested) *tris_tested = nt;
    return 0;
}

// ---- a walk of the package's CWBVH (test infrastructure) -------------------------------------
// A host restatement of the device traversal of one ray (merian_gb300/csrc/device_scene.cuh:
// set_ray, intersect_node, trace_loop in the per-thread order, i.e. without postponed triangle
// groups) over the 80-byte nodes and 48-byte triangle records gbpt_bvh_build returns, for
// single-level trees. Every box-test operation is rounded once in the device's order
// (__fmul_rn / __fsub_rn / __fmaf_rn there, -ffp-contract=off and std::fma here), so the walk
// makes the same box decisions: it visits the same nodes and tests the same triangles as the
// device, and finds the same closest (or any) hit with the watertight test above. It gives the
// node and triangle counts per ray of the roofline's algorithmic bytes.
namespace oracle {
namespace cw {
constexpr float kErr = 1.0f / 1048576.0f, kBiasErr = 1.0f / 256.0f, kPlaneBias = 32768.0f;
inline float bits_f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline uint32_t f_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
// the device's byte permute: byte j of w in bits 8..15 of the float 32768.0
inline float qplane(uint32_t w, int j) { return bits_f(0x47000000u | (((w >> (8 * j)) & 0xFFu) << 8)); }

struct Walk {
    const uint32_t* nodes; // 20 words per node
    const float* tris;     // 12 floats per record
    float o[3], inv[3], tmin;
    uint32_t oct_inv, oct_inv4;
    bool neg[3];
    RayPre<float> pre;
    float best_t, best_u, best_v;
    uint32_t best_prim, best_geom;
    bool found;
};

inline uint32_t intersect_node(const Walk& w, uint32_t ni, uint32_t& cb, uint32_t& tb,
                               uint32_t& imask) {
    const uint32_t* n = w.nodes + 20ull * ni;
    float ai[3], no[3], fo[3];
    for (int k = 0; k < 3; ++k) {
        ai[k] = bits_f(((n[3] >> (8 * k)) & 0xFFu) << 23) * w.inv[k];
        const float ao = (bits_f(n[k]) - w.o[k]) * w.inv[k];
        const float e = std::fma(kBiasErr, std::fabs(ai[k]),
                                 std::fma(255.0f, std::fabs(ai[k]), std::fabs(ao)) * kErr);
        no[k] = std::fma(-kPlaneBias, ai[k], ao - e);
        fo[k] = std::fma(-kPlaneBias, ai[k], ao + e);
    }
    imask = n[3] >> 24;
    cb = n[4];
    tb = n[5];
    uint32_t hitmask = 0;
    for (int half = 0; half < 2; ++half) {
        const uint32_t meta4 = n[6 + half];
        const uint32_t is_inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
        const uint32_t inner_mask4 = (is_inner4 >> 4) * 0xFFu;
        const uint32_t bit_index4 = (meta4 ^ (w.oct_inv4 & inner_mask4)) & 0x1F1F1F1Fu;
        const uint32_t child_bits4 = (meta4 >> 5) & 0x07070707u;
        // planes: lo x, lo y, lo z, hi x, hi y, hi z words of this half
        const uint32_t ql[3] = {n[8 + half], n[10 + half], n[12 + half]};
        const uint32_t qh[3] = {n[14 + half], n[16 + half], n[18 + half]};
        for (int j = 0; j < 4; ++j) {
            float tn[3], tf[3];
            for (int k = 0; k < 3; ++k) {
                tn[k] = std::fma(qplane(w.neg[k] ? qh[k] : ql[k], j), ai[k], no[k]);
                tf[k] = std::fma(qplane(w.neg[k] ? ql[k] : qh[k], j), ai[k], fo[k]);
            }
            const float cmin = std::fmax(std::fmax(tn[0], tn[1]), std::fmax(tn[2], w.tmin));
            const float cmax = std::fmin(std::fmin(tf[0], tf[1]), std::fmin(tf[2], w.best_t));
            const uint32_t sh = 8u * j;
            if (cmin <= cmax) hitmask |= ((child_bits4 >> sh) & 7u) << ((bit_index4 >> sh) & 31u);
        }
    }
    return hitmask;
}

// one ray: adds the nodes visited and triangles tested to the counts
inline void walk_ray(Walk& w, const gbpt_ray& r, uint32_t mask, bool any_hit, uint64_t& nodes,
                     uint64_t& tris) {
    for (int k = 0; k < 3; ++k) {
        const float d = r.direction[k];
        w.o[k] = r.origin[k];
        w.inv[k] = 1.0f / (std::fabs(d) > 1e-20f ? d : std::copysign(1e-20f, d));
        w.neg[k] = (f_bits(d) >> 31) != 0u;
    }
    const uint32_t oct = (f_bits(r.direction[0]) >> 31) | ((f_bits(r.direction[1]) >> 31) << 1) |
                         ((f_bits(r.direction[2]) >> 31) << 2);
    w.oct_inv = 7u - oct;
    w.oct_inv4 = w.oct_inv * 0x01010101u;
    w.pre = ray_pre<float>(Ray<float>{mk<float>(r.origin[0], r.origin[1], r.origin[2]),
                                      mk<float>(r.direction[0], r.direction[1], r.direction[2]),
                                      r.tmin, r.tmax});
    w.tmin = r.tmin;
    w.best_t = r.tmax;
    w.best_u = w.best_v = 0.0f;
    w.best_prim = w.best_geom = kNoInst;
    w.found = false;
    uint32_t ng[2] = {0u, 0x80000000u}, tg[2] = {0u, 0u};
    std::vector<std::array<uint32_t, 2>> stack;
    while (true) {
        if (ng[1] > 0x00FFFFFFu) {
            const uint32_t hits = ng[1];
            const uint32_t bit = 31u - (uint32_t)__builtin_clz(hits & 0xFF000000u);
            ng[1] &= ~(1u << bit);
            if (ng[1] > 0x00FFFFFFu) stack.push_back({ng[0], ng[1]});
            const uint32_t slot = (bit - 24u) ^ w.oct_inv;
            const uint32_t ni =
                ng[0] + (uint32_t)__builtin_popcount((hits & 0xFFu) & ((1u << slot) - 1u));
            uint32_t cb, tb, im;
            ++nodes;
            const uint32_t hm = intersect_node(w, ni, cb, tb, im);
            ng[0] = cb;
            ng[1] = (hm & 0xFF000000u) | im;
            tg[0] = tb;
            tg[1] = hm & 0x00FFFFFFu;
        } else {
            tg[0] = ng[0];
            tg[1] = ng[1];
            ng[0] = ng[1] = 0u;
        }
        bool done = false;
        while (tg[1] != 0u) {
            const uint32_t b = (uint32_t)__builtin_ctz(tg[1]);
            tg[1] &= tg[1] - 1u;
            const float* rec = w.tris + 12ull * (tg[0] + b);
            const uint32_t tfl = f_bits(rec[11]);
            if (((tfl & 0xFFu) & mask) == 0u) continue;
            ++tris;
            const float tv[9] = {rec[0], rec[1], rec[2], rec[4], rec[5], rec[6], rec[8], rec[9],
                                 rec[10]};
            const uint32_t flags = ((tfl & (1u << 8)) ? GBPT_MESH_TWO_SIDED : 0u) |
                                   ((tfl & (1u << 9)) ? GBPT_MESH_FLIP_FACING : 0u);
            float t, u, v;
            if (!intersect<float>(w.pre, tv, flags, w.tmin, w.best_t, t, u, v)) continue;
            const uint32_t prim = f_bits(rec[3]), geom = f_bits(rec[7]);
            if (t < w.best_t || geom < w.best_geom || (geom == w.best_geom && prim < w.best_prim)) {
                w.best_t = t;
                w.best_u = u;
                w.best_v = v;
                w.best_prim = prim;
                w.best_geom = geom;
                w.found = true;
                if (any_hit) {
                    done = true;
                    break;
                }
            }
        }
        if (done) break;
        if (ng[1] <= 0x00FFFFFFu) {
            if (stack.empty()) break;
            ng[0] = stack.back()[0];
            ng[1] = stack.back()[1];
            stack.pop_back();
        }
    }
}
} // namespace cw
} // namespace oracle

// Closest (or any) hits of n rays through a single-level CWBVH of gbpt_bvh_build (node and
// triangle arrays as it returns them), in the gbpt_hit layout of the device's gbpt_trace, and per
// ray the nodes visited and triangles tested (counts_out: 2 per ray, may be null).
ORACLE_API int oracle_cwbvh_trace(const void* nodes, uint64_t n_nodes, const void* tris,
                                  uint64_t n_tris, const gbpt_ray* rays, uint32_t n, uint32_t mask,
                                  int any_hit, gbpt_hit* out, uint32_t* counts_out) {
    using namespace oracle;
    if (!nodes || !n_nodes || !tris || !rays || !out) return -1;
    (void)n_tris;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        cw::Walk w;
        w.nodes = (const uint32_t*)nodes;
        w.tris = (const float*)tris;
        uint64_t a = 0, b = 0;
        cw::walk_ray(w, rays[i], mask & 0xFFu, any_hit != 0, a, b);
        gbpt_hit& h = out[i];
        const bool ok = w.found;
        h.instance_id = ok ? 0u : kNoInst;
        h.instance_index = ok ? 0u : kNoInst;
        h.primitive_id = ok ? w.best_prim : kNoInst;
        h.geometry_index = ok ? w.best_geom : kNoInst;
        h.barycentrics[0] = ok ? w.best_u : 0.f;
        h.barycentrics[1] = ok ? w.best_v : 0.f;
        h.t = ok ? w.best_t : -1.0f;
        h.reserved = 0;
        if (counts_out) {
            counts_out[2 * i] = (uint32_t)a;
            counts_out[2 * i + 1] = (uint32_t)b;
        }
    }
    return 0;
}

// ---- the path tracer ------------------------------------------------------------------------
namespace oracle {

struct PathCfg {
    int max_path_length;
    bool emission_on_primary;
    uint32_t mask;
    bool nee;
    int rr_depth;
};

struct PathCounters {
    uint64_t rays = 0;
    // when set, the closest-hit bounce rays (path segments 2..L, not camera or shadow rays)
    std::vector<gbpt_ray>* bounce = nullptr;
};

template <class R> struct LightSample {
    V3<R> dir;    // towards the light
    R dist;       // shadow ray length
    V3<R> le;     // emitted radiance
    R pdf;        // solid angle, including selection
    bool valid;
};

// Selection: environment with probability 1/2 when both kinds exist.
template <class R> inline R env_select_prob(const Scene& s) {
    if (s.ew == 0) return R(0);
    return s.light_tri.empty() ? R(1) : R(0.5);
}

template <class R> inline R env_pdf(const Scene& s, V3<R> dir) {
    if (s.ew == 0) return R(0);
    const float* M = s.env_to_local;
    const V3<R> l = normalize(mk<R>((R)M[0] * dir.x + (R)M[1] * dir.y + (R)M[2] * dir.z,
                                    (R)M[3] * dir.x + (R)M[4] * dir.y + (R)M[5] * dir.z,
                                    (R)M[6] * dir.x + (R)M[7] * dir.y + (R)M[8] * dir.z));
    const R u = std::atan2(l.x, -l.z) * C<R>::INV_2PI + R(0.5);
    const R v = std::acos(clampr(l.y, R(-1), R(1))) * C<R>::INV_PI;
    const R st = std::sin(v * C<R>::PI);
    if (!(st > R(0))) return R(0);
    uint32_t x = (uint32_t)std::min<double>(std::max<double>(std::floor(u * s.ew), 0.0), s.ew - 1);
    uint32_t y = (uint32_t)std::min<double>(std::max<double>(std::floor(v * s.eh), 0.0), s.eh - 1);
    const R pdf_uv = (R)(s.env_func[(size_t)y * s.ew + x] / s.env_func_int);
    return pdf_uv / (R(2) * C<R>::PI * C<R>::PI * st);
}

inline uint32_t global_tri(const Scene& s, uint32_t geom, uint32_t prim) {
    return s.geom_tri_base[geom] + prim;
}

// World-space vertices of a hit triangle (object vertices placed by the hit's instance).
template <class R>
inline void world_tri(const Scene& s, uint32_t geom, uint32_t prim, uint32_t inst, V3<R> v[3]) {
    const gbpt_geometry& g = s.geoms[geom];
    const uint32_t tri = g.first_triangle + prim;
    for (int c = 0; c < 3; ++c) {
        const float* p = s.verts[g.first_vertex + s.idx[3 * tri + c]].position;
        if (inst == kNoInst) {
            v[c] = mk<R>(p[0], p[1], p[2]);
        } else {
            const float* r = s.insts[inst].o2w;
            float w[3];
            for (int a = 0; a < 3; ++a)
                w[a] = (float)((double)r[4 * a] * p[0] + (double)r[4 * a + 1] * p[1] +
                               (double)r[4 * a + 2] * p[2] + (double)r[4 * a + 3]);
            v[c] = mk<R>(w[0], w[1], w[2]);
        }
    }
}

// solid-angle pdf of reaching a point of the emissive world-space triangle (a, b, c) of geometry
// geom at squared distance dist2 along dir (from the shading point towards the light)
template <class R>
inline R tri_light_pdf(const Scene& s, const V3<R> tri[3], uint32_t geom, R dist2, V3<R> dir) {
    const gbpt_geometry& g = s.geoms[geom];
    const V3<R> n = normalize(cross(tri[1] - tri[0], tri[2] - tri[0]));
    const R cos_l = dot(dir, n);
    const gbpt_material& m = s.mats[g.material_id];
    const R lum = (R)(0.299 * m.emission[0] + 0.587 * m.emission[1] + 0.114 * m.emission[2]);
    const R area = R(0.5) * length(cross(tri[1] - tri[0], tri[2] - tri[0]));
    const R pmf = area * lum / (R)s.light_total;
    return (R(1) - env_select_prob<R>(s)) * pmf / area * dist2 / std::fabs(cos_l);
}

template <class R, class G>
LightSample<R> sample_light(const Scene& s, V3<R> pos, G& rng) {
    LightSample<R> ls{};
    ls.valid = false;
    const R u0 = rng.next_float(), u1 = rng.next_float(), u2 = rng.next_float();
    const R pe = env_select_prob<R>(s);
    if (pe <= R(0) && s.light_tri.empty()) return ls;
    if (u0 < pe) {
        // environment: row by the marginal, column by the conditional
        const double tr = (double)u1 * s.env_marg[s.eh];
        uint32_t y = (uint32_t)(std::upper_bound(s.env_marg.begin() + 1, s.env_marg.end(), tr) -
                                (s.env_marg.begin() + 1));
        y = std::min(y, s.eh - 1);
        const double* c = &s.env_cond[(size_t)y * (s.ew + 1)];
        const double tc = (double)u2 * c[s.ew];
        uint32_t x = (uint32_t)(std::upper_bound(c + 1, c + s.ew + 1, tc) - (c + 1));
        x = std::min(x, s.ew - 1);
        const double fy = (tr - s.env_marg[y]) / (s.env_marg[y + 1] - s.env_marg[y]);
        const double fx = (tc - c[x]) / (c[x + 1] - c[x]);
        const R u = (R)((x + std::min(std::max(fx, 0.0), 1.0)) / s.ew);
        const R v = (R)((y + std::min(std::max(fy, 0.0), 1.0)) / s.eh);
        // latlong_map_to_world (utils/math.slang:254-260), then back to world by to_local^T
        const R phi = C<R>::PI * (R(2) * u - R(1)), theta = C<R>::PI * v;
        const R st = std::sin(theta);
        const V3<R> dl = mk(st * std::sin(phi), std::cos(theta), -st * std::cos(phi));
        const float* M = s.env_to_local;
        const V3<R> dw = mk<R>((R)M[0] * dl.x + (R)M[3] * dl.y + (R)M[6] * dl.z,
                               (R)M[1] * dl.x + (R)M[4] * dl.y + (R)M[7] * dl.z,
                               (R)M[2] * dl.x + (R)M[5] * dl.y + (R)M[8] * dl.z);
        ls.dir = normalize(dw);
        ls.dist = R(1e7f);
        ls.le = env_eval(s, ls.dir);
        ls.pdf = pe * env_pdf(s, ls.dir);
        ls.valid = ls.pdf > R(0);
        return ls;
    }
    // emissive triangle by power, uniform point (sample_triangle, utils/sampling.slang:31-36)
    const double ut = pe > R(0) ? (double)((u0 - pe) / (R(1) - pe)) : (double)u0;
    size_t k = (size_t)(std::upper_bound(s.light_cdf.begin(), s.light_cdf.end(), ut) -
                        s.light_cdf.begin());
    k = std::min(k, s.light_tri.size() - 1);
    const uint32_t tri = s.light_tri[k];
    const R x = std::sqrt(u1);
    const R b0 = R(1) - x, b1 = x * (R(1) - u2), b2 = x * u2;
    const float* lt = &s.light_tv[9 * (size_t)tri];
    const V3<R> a = mk<R>(lt[0], lt[1], lt[2]);
    const V3<R> b = mk<R>(lt[3], lt[4], lt[5]);
    const V3<R> c = mk<R>(lt[6], lt[7], lt[8]);
    const V3<R> pl = (b0 * a + b1 * b) + b2 * c;
    V3<R> n = normalize(cross(b - a, c - a));
    const gbpt_geometry& g = s.geoms[s.light_geom[tri]];
    if (g.flags & GBPT_MESH_FLIP_FACING) n = -n;
    const V3<R> d = pl - pos;
    const R dist2 = dot(d, d);
    const R dist = std::sqrt(dist2);
    ls.dir = d / dist;
    const R cos_l = -dot(ls.dir, n);
    if (!(cos_l > R(0)) || !(dist > R(0))) return ls; // back of a one-sided emitter
    const gbpt_material& m = s.mats[g.material_id];
    ls.le = mk<R>(m.emission[0], m.emission[1], m.emission[2]);
    ls.dist = dist * R(1 - 1e-4f);
    const V3<R> wt[3] = {a, b, c};
    ls.pdf = tri_light_pdf<R>(s, wt, s.light_geom[tri], dist2, ls.dir);
    ls.valid = ls.pdf > R(0);
    return ls;
}

// One sample of trace_path (render_pt.slang:24-90); with cfg.nee/rr the GB300 estimator (NEE with
// power-heuristic MIS, Russian roulette), which has the same expectation.
template <class R>
V3<R> trace_path(const Scene& s, const PathCfg& cfg, Ray<R> ray, SP<R> sp, Pcg& rng,
                 PathCounters& ctr) {
    R current_ior = R(1);
    V3<R> throughput = mk(R(1), R(1), R(1));
    V3<R> radiance = cfg.emission_on_primary ? throughput * sp.emission : mk(R(0), R(0), R(0));
    const R thr = R(1e-5f); // SCENE_THROUGHPUT_THRESHOLD (scene.slang:24)
    for (int bounce = 1; bounce < cfg.max_path_length; ++bounce) {
        if (!sp.has_material ||
            (throughput.x < thr && throughput.y < thr && throughput.z < thr))
            break;
        if (cfg.rr_depth > 0 && bounce >= cfg.rr_depth) {
            const R q = minr(R(1), maxr(throughput.x, maxr(throughput.y, throughput.z)));
            if ((R)rng.next_float() >= q) break;
            throughput = throughput / q;
        }
        const Frame<R>& frame = sp.frame;
        const V3<R> wi_local = frame.to_local(-ray.d);
        const V3<R> ng = decode_normal<R>(sp.enc_face_normal);
        if (cfg.nee) {
            const LightSample<R> ls = sample_light(s, sp.pos, rng);
            if (ls.valid) {
                const V3<R> wl_local = frame.to_local(ls.dir);
                const bool trans = wi_local.z * wl_local.z < R(0);
                const R wl_ng = dot(ls.dir, ng);
                const bool geo_ok = ((dot(-ray.d, ng) < R(0)) != (wl_ng < R(0))) == trans;
                if (geo_ok) {
                    const V3<R> f = sp.bsdf.eval(wi_local, wl_local);
                    const R pb = sp.bsdf.pdf(wi_local, wl_local);
                    if (f.x > R(0) || f.y > R(0) || f.z > R(0)) {
                        Ray<R> sr;
                        sr.o = offset_ray_origin(sp.pos, wl_ng < R(0) ? -ng : ng);
                        sr.d = ls.dir;
                        sr.tmin = R(0);
                        sr.tmax = ls.dist;
                        ctr.rays++;
                        const HitRec occ = trace<R>(s, sr, cfg.mask, true);
                        if (!occ.valid) {
                            const R wmis = power_heuristic(ls.pdf, pb);
                            radiance = radiance + throughput * f * ls.le * (wmis / ls.pdf);
                        }
                    }
                }
            }
        }
        const Sample<R> bs = sp.bsdf.sample_eval(wi_local, rng);
        if (!bs.valid) break;
        const V3<R> wo = frame.to_world(bs.wo);
        throughput = throughput * bs.weight;
        const bool transmission = wi_local.z * bs.wo.z < R(0);
        if (transmission) current_ior = current_ior / sp.bsdf.eta;
        // make_ray (hit.slang:134-146)
        const R wo_ng = dot(wo, ng);
        if (((dot(-ray.d, ng) < R(0)) != (wo_ng < R(0))) != transmission) break;
        ray.o = offset_ray_origin(sp.pos, wo_ng < R(0) ? -ng : ng);
        ray.d = wo;
        ray.tmin = R(0);
        ray.tmax = R(1e7f);
        ctr.rays++;
        if (ctr.bounce) {
            gbpt_ray g{};
            g.origin[0] = (float)ray.o.x;
            g.origin[1] = (float)ray.o.y;
            g.origin[2] = (float)ray.o.z;
            g.direction[0] = (float)ray.d.x;
            g.direction[1] = (float)ray.d.y;
            g.direction[2] = (float)ray.d.z;
            g.tmin = (float)ray.tmin;
            g.tmax = (float)ray.tmax;
            ctr.bounce->push_back(g);
        }
        const HitRec h = trace<R>(s, ray, cfg.mask, false);
        sp = shading_point<R>(s, ray, h, current_ior, bounce + 1 < cfg.max_path_length, false);
        V3<R> e = throughput * sp.emission;
        if (cfg.nee && (e.x != R(0) || e.y != R(0) || e.z != R(0))) {
            R pl = R(0);
            if (!h.valid || (s.geoms[h.geom].flags & GBPT_MESH_USE_ENV_MAP)) {
                pl = env_select_prob<R>(s) * env_pdf(s, ray.d);
            } else if (sp.emissive_tri) {
                V3<R> wt[3];
                world_tri<R>(s, h.geom, h.prim, h.inst, wt);
                pl = tri_light_pdf<R>(s, wt, h.geom, pow2((R)h.t), ray.d);
            }
            e = e * power_heuristic(bs.pdf, pl);
        }
        radiance = radiance + e;
    }
    return radiance;
}

// raygen main (render_pt.slang:92-130) for one pixel: returns the per-frame output (mean rgb,
// mean luminance^2) and, for the statistical parity tests, the per-sample rgb sum of squares.
template <class R>
void render_pixel(const Scene& s, const gbpt_camera& cam, const gbpt_render_params& p,
                  const PathCfg& cfg, uint32_t px, uint32_t py, double* rgba, double* sq,
                  double* lum4, PathCounters& ctr) {
    const Ray<R> primary = camera_ray<R>(cam, px, py, p.width, p.height);
    ctr.rays++;
    const HitRec h = trace<R>(s, primary, cfg.mask, false);
    const SP<R> psp = shading_point<R>(s, primary, h, R(1), true, true);
    // "demodulate albedo" (render_pt.slang:105-116): every sample divided by the GBuffer albedo
    // floored at 1e-2 (gbuffer.slang:135-140), taken at the full-precision hit
    V3<R> demod = mk(R(1), R(1), R(1));
    if (p.demodulate_albedo) {
        const SP<R> g = shading_point<R>(s, primary, h, R(1), true, false);
        const V3<R> a = g.has_material ? g.bsdf.get_albedo(g.frame.to_local(-primary.d)) : g.emission;
        demod = mk(maxr(a.x, R(1e-2f)), maxr(a.y, R(1e-2f)), maxr(a.z, R(1e-2f)));
    }
    double acc[3] = {0, 0, 0}, sm = 0.0, s2[3] = {0, 0, 0}, s4 = 0.0;
    for (int smp = 0; smp < p.spp; ++smp) {
        Pcg rng{pcg4d16(px, py, p.frame, (uint32_t)smp)};
        const V3<R> c = trace_path<R>(s, cfg, primary, psp, rng, ctr) / demod;
        if (!(std::isfinite((double)c.x) && std::isfinite((double)c.y) &&
              std::isfinite((double)c.z)))
            continue;
        acc[0] += (double)c.x;
        acc[1] += (double)c.y;
        acc[2] += (double)c.z;
        s2[0] += (double)c.x * (double)c.x;
        s2[1] += (double)c.y * (double)c.y;
        s2[2] += (double)c.z * (double)c.z;
        const double l = (double)yuv_luminance(c);
        sm += l * l;
        s4 += (l * l) * (l * l);
    }
    const double inv = p.spp > 0 ? 1.0 / p.spp : 0.0;
    rgba[0] = acc[0] * inv;
    rgba[1] = acc[1] * inv;
    rgba[2] = acc[2] * inv;
    rgba[3] = sm * inv;
    if (sq) {
        sq[0] = s2[0] * inv;
        sq[1] = s2[1] * inv;
        sq[2] = s2[2] * inv;
    }
    // the second moment of the `a` channel's samples: its variance is E[l^4] - E[l^2]^2
    if (lum4) *lum4 = s4 * inv;
}

} // namespace oracle

// Renders the listed pixels (or all) at p->spp. out_rgba: 4 doubles per pixel (mean rgb, mean
// luminance^2); out_sq (optional): 3 doubles per pixel, mean of the squared per-sample rgb;
// out_lum4 (optional): 1 double per pixel, mean of luminance^4. threads <= 0 uses every host
// thread. Returns the number of traced rays in *out_rays.
ORACLE_API int oracle_render(void* sp, const gbpt_camera* cam, const gbpt_render_params* p,
                             int fp64, int threads, double* out_rgba, double* out_sq,
                             double* out_lum4, uint64_t* out_rays) {
    const Scene& s = *(const Scene*)sp;
    PathCfg cfg{p->max_path_length, p->emission_on_primary != 0, p->instance_mask & 0xFFu,
                p->nee != 0, p->rr_depth};
    const uint32_t n = p->pixel_count ? p->pixel_count : p->width * p->height;
    std::atomic<uint64_t> rays{0};
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
#pragma omp parallel
    {
        PathCounters ctr;
#pragma omp for schedule(dynamic, 1)
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            const uint32_t pix = p->pixel_count ? p->pixels[i] : (uint32_t)i;
            const uint32_t px = pix % p->width, py = pix / p->width;
            double* sq = out_sq ? out_sq + 3 * i : nullptr;
            double* l4 = out_lum4 ? out_lum4 + i : nullptr;
            if (fp64)
                render_pixel<double>(s, *cam, *p, cfg, px, py, out_rgba + 4 * i, sq, l4, ctr);
            else
                render_pixel<float>(s, *cam, *p, cfg, px, py, out_rgba + 4 * i, sq, l4, ctr);
        }
        rays += ctr.rays;
    }
    if (out_rays) *out_rays = rays;
    return 0;
}

// The closest-hit bounce rays (segments 2..L of every path) the FP32 build traces for the listed
// pixels at p->spp: a sample of a workload's bounce-ray distribution. Writes up to `cap` rays,
// in pixel order, and their number in *n_out (the total, which may exceed cap).
ORACLE_API int oracle_bounce_rays(void* sp, const gbpt_camera* cam, const gbpt_render_params* p,
                                  gbpt_ray* out, uint64_t cap, uint64_t* n_out) {
    const Scene& s = *(const Scene*)sp;
    PathCfg cfg{p->max_path_length, p->emission_on_primary != 0, p->instance_mask & 0xFFu,
                p->nee != 0, p->rr_depth};
    const uint32_t n = p->pixel_count ? p->pixel_count : p->width * p->height;
    std::vector<std::vector<gbpt_ray>> per(n);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const uint32_t pix = p->pixel_count ? p->pixels[i] : (uint32_t)i;
        PathCounters ctr;
        ctr.bounce = &per[i];
        double rgba[4];
        render_pixel<float>(s, *cam, *p, cfg, pix % p->width, pix / p->width, rgba, nullptr,
                            nullptr, ctr);
    }
    uint64_t k = 0;
    for (const auto& v : per)
        for (const gbpt_ray& r : v) {
            if (k < cap && out) out[k] = r;
            ++k;
        }
    if (n_out) *n_out = k;
    return 0;
}

// FP32 primary shading points in the layout of gbpt_debug_primary_points (24 floats per pixel).
ORACLE_API int oracle_primary_points(void* sp, const gbpt_camera* cam, const gbpt_render_params* p,
                                     float* out) {
    const Scene& s = *(const Scene*)sp;
    const uint32_t n = p->pixel_count ? p->pixel_count : p->width * p->height;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t pix = p->pixel_count ? p->pixels[i] : i;
        const Ray<float> r = camera_ray<float>(*cam, pix % p->width, pix / p->width, p->width,
                                               p->height);
        const HitRec h = trace<float>(s, r, p->instance_mask & 0xFFu, false);
        const SP<float> q = shading_point<float>(s, r, h, 1.0f, true, true);
        float* o = out + 24ull * i;
        const uint32_t mat = h.valid ? s.geoms[h.geom].material_id : 0u;
        const uint32_t fl = (q.has_material ? 1u : 0u) |
                            (q.front ? 2u : 0u);
        const float v[24] = {q.pos.x, q.pos.y, q.pos.z, as_float(q.enc_face_normal),
                             q.frame.n.x, q.frame.n.y, q.frame.n.z, as_float(mat),
                             q.frame.t.x, q.frame.t.y, q.frame.t.z, as_float(fl),
                             q.frame.b.x, q.frame.b.y, q.frame.b.z, 0.f,
                             q.emission.x, q.emission.y, q.emission.z, 0.f,
                             r.d.x, r.d.y, r.d.z, 0.f};
        std::memcpy(o, v, sizeof(v));
    }
    return 0;
}

// The GBuffer (Raytraced) node for a static camera (gbuffer_rt.slang:18-94, gbuffer.slang:40-160)
// in FP32: per pixel one gbpt_gbuffer_texel. Motion vectors are 0 and delta_z is
// |pos - camera| - linear_z (0): the previous camera and transforms equal the current ones.
ORACLE_API int oracle_gbuffer(void* sp, const gbpt_camera* cam, uint32_t w, uint32_t h,
                              uint32_t mask, gbpt_gbuffer_texel* out) {
    using R = float;
    const Scene& s = *(const Scene*)sp;
    const V3<R> U = mk<R>(cam->U[0], cam->U[1], cam->U[2]), V = mk<R>(cam->V[0], cam->V[1], cam->V[2]),
                W = mk<R>(cam->W[0], cam->W[1], cam->W[2]);
    const V3<R> cpos = mk<R>(cam->position[0], cam->position[1], cam->position[2]);
    auto pinhole = [&](uint32_t px, uint32_t py) { // camera.slang:34-37
        const R x = ((R)px + R(0.5) + (R)cam->jitter[0]) / (R)w;
        const R y = ((R)py + R(0.5) + (R)cam->jitter[1]) / (R)h;
        return normalize((R(2) * x + R(-1)) * U + (R(-2) * y + R(1)) * V + W);
    };
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)w * h; ++i) {
        const uint32_t px = (uint32_t)(i % w), py = (uint32_t)(i / w);
        const Ray<R> r = camera_ray<R>(*cam, px, py, w, h);
        const HitRec hr = trace<R>(s, r, mask & 0xFFu, false);
        gbpt_gbuffer_texel t{};
        gbpt_hit ph;
        fill_hit<float>(s, hr, ph);
        t.instance_id = ph.instance_id;
        t.primitive_id = ph.primitive_id;
        t.geometry_index = (uint16_t)ph.geometry_index;
        t.instance_index = (uint16_t)ph.instance_index;
        t.barycentrics = hr.valid ? ((uint32_t)float_to_half(hr.v) << 16) | float_to_half(hr.u) : 0u;
        const bool env = !hr.valid || (s.geoms[hr.geom].flags & GBPT_MESH_USE_ENV_MAP);
        if (env) {
            const SP<R> e = env_sp<R>(s, r);
            t.encoded_normal = encode_normal(e.frame.n.x, e.frame.n.y, e.frame.n.z);
            t.linear_z = std::min(length(e.pos - r.o), 65504.0f);
            for (int c = 0; c < 3; ++c) {
                t.albedo[c] = (&e.emission.x)[c];
                t.emission[c] = (&e.emission.x)[c];
            }
        } else {
            const SP<R> q = shading_point<R>(s, r, hr, R(1), true, false);
            const gbpt_geometry& g = s.geoms[hr.geom];
            const uint32_t tri = g.first_triangle + hr.prim;
            V3<R> p0 = fetch_pos<R>(s, g.first_vertex + s.idx[3 * tri + 0]);
            V3<R> p1 = fetch_pos<R>(s, g.first_vertex + s.idx[3 * tri + 1]);
            V3<R> p2 = fetch_pos<R>(s, g.first_vertex + s.idx[3 * tri + 2]);
            V3<R> e1 = p1 - p0, e2 = p2 - p0;
            if (hr.inst != kNoInst) {
                e1 = xform_vector<R>(s.insts[hr.inst].o2w, e1);
                e2 = xform_vector<R>(s.insts[hr.inst].o2w, e2);
            }
            V3<R> fn = normalize(cross(e1, e2));
            if (g.flags & GBPT_MESH_FLIP_FACING) fn = -fn;
            const R lz = length(q.pos - r.o);
            // Surface::compute_grad_z (hit.slang:99-103)
            const R n_dot_oo = dot(fn, q.pos - r.o);
            const R gx = n_dot_oo / dot(fn, pinhole(px + 1, py)) - lz;
            const R gy = n_dot_oo / dot(fn, pinhole(px, py + 1)) - lz;
            t.grad_z = ((uint32_t)float_to_half(gy) << 16) | float_to_half(gx);
            t.encoded_normal = encode_normal(q.frame.n.x, q.frame.n.y, q.frame.n.z);
            t.linear_z = std::min(lz, 65504.0f);
            t.delta_z = length(q.pos - cpos) - lz;
            const V3<R> a = q.bsdf.get_albedo(q.frame.to_local(-r.d));
            t.albedo[0] = a.x;
            t.albedo[1] = a.y;
            t.albedo[2] = a.z;
            t.emission[0] = q.emission.x;
            t.emission[1] = q.emission.y;
            t.emission[2] = q.emission.z;
        }
        out[i] = t;
    }
    return 0;
}

// The pinhole camera basis of merian's Camera (camera.cpp:263-266 recompute_ray_basis,
// :349-367 write_to), in float as the host computes it: forward = normalize(target - position),
// right = normalize(cross(forward, up)), focus = |target - position|, h = tan(vfov / 2);
// U = right * h * aspect * focus, V = cross(right, forward) * h * focus, W = forward * focus.
// The oracle's own restatement, so the CPU baseline and the fixtures can set up a camera
// without the product library.
ORACLE_API int oracle_camera_look_at(const float* position, const float* target, const float* up,
                                     float vfov, float aspect, float near_plane, float far_plane,
                                     gbpt_camera* out) {
    using namespace oracle;
    if (!position || !target || !up || !out) return -1;
    const V3<float> o = mk(position[0], position[1], position[2]);
    const V3<float> to_target = mk(target[0], target[1], target[2]) - o;
    const V3<float> forward = normalize(to_target);
    const V3<float> right = normalize(cross(forward, mk(up[0], up[1], up[2])));
    const float focus = std::sqrt(dot(to_target, to_target));
    const float h = std::tan(vfov * 0.5f);
    const V3<float> basis[4] = {o, (h * aspect * focus) * right,
                                (h * focus) * cross(right, forward), focus * forward};
    std::memset(out, 0, sizeof(*out));
    float* dst[4] = {out->position, out->U, out->V, out->W};
    for (int k = 0; k < 4; ++k) {
        dst[k][0] = basis[k].x;
        dst[k][1] = basis[k].y;
        dst[k][2] = basis[k].z;
    }
    out->near_plane = near_plane;
    out->far_plane = far_plane;
    return 0;
}

// The scene generators compiled into this library report argument errors through
// gbpt::set_error; here the message is kept for oracle_last_error.
namespace gbpt {
static thread_local std::string g_oracle_error;
void set_error(const std::string& msg) { g_oracle_error = msg; }
} // namespace gbpt
ORACLE_API const char* oracle_last_error(void) { return gbpt::g_oracle_error.c_str(); }

// The alias-table builder the package compiles into scene upload (host_common.h), for the tests
// that check the kernels' environment sampling against the density it encodes.
ORACLE_API void oracle_alias_table(const double* w, uint32_t n, uint32_t* out) {
    gbpt::alias_table(w, n, out);
}

ORACLE_API int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// ---- BSDF property checks (tests/bsdf/bsdf-checks.slang:30-135) -----------------------------
// kind: 0 Lambert(albedo), 1 GGX(alpha, alpha_y), 2 Conductor(alpha, f0), 3 RoughDielectric(alpha,
// eta = 1/1.5, tint = albedo), 4 FresnelMix<GGX, Lambert>(alpha, albedo, ior_f0). out: 16 floats in
// the reference's slot layout (furnace rgb, furnace stderr rgb, mean_cos, stderr_cos, valid,
// max_weight_err, max_pdf_err, pdf_integral, max_recip_err, -, -, -).
// Consistency of a BSDF's evaluation with its sampler, the property next-event estimation and MIS
// rely on: out = {mean sample weight (furnace, r channel), full-sphere quadrature of eval (r),
// fraction of valid samples, full-sphere quadrature of pdf}. kind as oracle_bsdf_check.
ORACLE_API int oracle_bsdf_integrals(int kind, const double* wi_in, double alpha, double eta,
                                     double ior_f0, uint32_t n_samples, uint32_t n_theta,
                                     double* out) {
    using R = double;
    const V3<R> wi = mk(wi_in[0], wi_in[1], wi_in[2]);
    const V3<R> alb = mk(0.7, 0.7, 0.7);
    Lambert<R> lam{alb};
    GGX<R> ggx{alpha, alpha};
    Conductor<R> cond{GGX<R>{alpha, alpha}, mk(0.95, 0.64, 0.54)};
    RoughDielectric<R> rd{alpha, eta, mk(1.0, 1.0, 1.0)};
    OpaqueDielectric<R> fm{GGX<R>{alpha, alpha}, Lambert<R>{alb}, ior_f0};
    auto se = [&](XorShift& rng) -> Sample<R> {
        switch (kind) {
        case 0: return lam.sample_eval(wi, rng);
        case 1: return ggx.sample_eval(wi, rng);
        case 2: return cond.sample_eval(wi, rng);
        case 3: return rd.sample_eval(wi, rng);
        default: return fm.sample_eval(wi, rng);
        }
    };
    auto ev = [&](V3<R> wo) -> R {
        switch (kind) {
        case 0: return lam.eval(wi, wo).x;
        case 1: return ggx.eval(wi, wo).x;
        case 2: return cond.eval(wi, wo).x;
        case 3: return rd.eval(wi, wo).x;
        default: return fm.eval(wi, wo).x;
        }
    };
    auto pd = [&](V3<R> wo) -> R {
        switch (kind) {
        case 0: return lam.pdf(wi, wo);
        case 1: return ggx.pdf(wi, wo);
        case 2: return cond.pdf(wi, wo);
        case 3: return rd.pdf(wi, wo);
        default: return fm.pdf(wi, wo);
        }
    };
    XorShift rng{0x1234567u};
    double fur = 0.0;
    uint32_t valid = 0;
    for (uint32_t i = 0; i < n_samples; ++i) {
        const Sample<R> s = se(rng);
        if (s.valid) {
            fur += s.weight.x;
            ++valid;
        }
    }
    const uint32_t n_phi = 2 * n_theta;
    double ie = 0.0, ip = 0.0;
    for (uint32_t ti = 0; ti < n_theta; ++ti) {
        const double t = (ti + 0.5) * C<R>::PI / n_theta;
        const double st = std::sin(t), ct = std::cos(t);
        for (uint32_t pi = 0; pi < n_phi; ++pi) {
            const double p = (pi + 0.5) * C<R>::TWO_PI / n_phi;
            const V3<R> wo = mk(st * std::cos(p), st * std::sin(p), ct);
            const double dw = st * (C<R>::PI / n_theta) * (C<R>::TWO_PI / n_phi);
            ie += ev(wo) * dw;
            ip += pd(wo) * dw;
        }
    }
    out[0] = fur / n_samples;
    out[1] = ie;
    out[2] = (double)valid / n_samples;
    out[3] = ip;
    return 0;
}

// n samples of a material at one shading point, 12 floats each (wo, pdf, weight, valid, eval,
// pdf at wo); sample i draws from PCG(pcg4d16(i, seed, 0, 0)), as gbpt_debug_material_samples.
ORACLE_API int oracle_material_samples(const gbpt_material* m, int front, float ior,
                                       const float* wi_in, uint32_t seed, uint32_t n, float* out) {
    using R = float;
    const MaterialBSDF<R> mb = make_material<R>(*m, mk(1.f, 1.f, 1.f), ior, front != 0);
    const V3<R> wi = mk(wi_in[0], wi_in[1], wi_in[2]);
    for (uint32_t i = 0; i < n; ++i) {
        Pcg rng{pcg4d16(i, seed, 0u, 0u)};
        const Sample<R> s = mb.sample_eval(wi, rng);
        float* o = out + 12ull * i;
        o[0] = s.wo.x;
        o[1] = s.wo.y;
        o[2] = s.wo.z;
        o[3] = s.pdf;
        o[4] = s.weight.x;
        o[5] = s.weight.y;
        o[6] = s.weight.z;
        o[7] = s.valid ? 1.f : 0.f;
        const V3<R> e = s.valid ? mb.eval(wi, s.wo) : mk(0.f, 0.f, 0.f);
        o[8] = e.x;
        o[9] = e.y;
        o[10] = e.z;
        o[11] = s.valid ? mb.pdf(wi, s.wo) : 0.f;
    }
    return 0;
}

ORACLE_API int oracle_bsdf_check(int kind, const float* wi_in, const float* albedo, float alpha,
                                 float alpha_y, const float* f0, float ior_f0, float eta,
                                 uint32_t n_samples, uint32_t seed, float* out) {
    using R = float;
    const V3<R> wi = mk(wi_in[0], wi_in[1], wi_in[2]);
    const V3<R> alb = mk(albedo[0], albedo[1], albedo[2]);
    Lambert<R> lam{alb};
    GGX<R> ggx{alpha, alpha_y};
    Conductor<R> cond{GGX<R>{alpha, alpha}, mk(f0[0], f0[1], f0[2])};
    RoughDielectric<R> rd{alpha, eta, alb};
    OpaqueDielectric<R> fm{GGX<R>{alpha, alpha}, Lambert<R>{alb}, ior_f0};
    auto sample_eval = [&](V3<R> w, XorShift& rng) -> Sample<R> {
        switch (kind) {
        case 0: return lam.sample_eval(w, rng);
        case 1: return ggx.sample_eval(w, rng);
        case 2: return cond.sample_eval(w, rng);
        case 3: return rd.sample_eval(w, rng);
        default: return fm.sample_eval(w, rng);
        }
    };
    auto evalf = [&](V3<R> a, V3<R> b) -> V3<R> {
        switch (kind) {
        case 0: return lam.eval(a, b);
        case 1: return ggx.eval(a, b);
        case 2: return cond.eval(a, b);
        case 3: return rd.eval(a, b);
        default: return fm.eval(a, b);
        }
    };
    auto pdff = [&](V3<R> a, V3<R> b) -> R {
        switch (kind) {
        case 0: return lam.pdf(a, b);
        case 1: return ggx.pdf(a, b);
        case 2: return cond.pdf(a, b);
        case 3: return rd.pdf(a, b);
        default: return fm.pdf(a, b);
        }
    };
    auto acc_err = [](R acc, R v) { return std::isfinite(v) ? std::max(acc, v) : 1e30f; };
    XorShift rng{seed | 1u};
    V3<R> mean_w = mk(0.f, 0.f, 0.f), m2_w = mk(0.f, 0.f, 0.f);
    R mean_cos = 0, m2_cos = 0, max_w_err = 0, max_pdf_err = 0;
    uint32_t valid = 0;
    for (uint32_t i = 0; i < n_samples; ++i) {
        V3<R> w = mk(0.f, 0.f, 0.f);
        R c = 0;
        const Sample<R> s = sample_eval(wi, rng);
        if (s.valid) {
            valid++;
            w = s.weight;
            c = s.wo.z / s.pdf;
            const R pref = pdff(wi, s.wo);
            const V3<R> eref = evalf(wi, s.wo);
            max_pdf_err = acc_err(max_pdf_err, std::fabs(s.pdf - pref) /
                                                   (std::max(std::fabs(s.pdf), std::fabs(pref)) +
                                                    1e-6f));
            if (pref > 0) max_w_err = acc_err(max_w_err, length(s.weight - eref / pref));
        }
        const R inv_i = 1.0f / (R)(i + 1);
        const V3<R> dw = w - mean_w;
        mean_w = mean_w + dw * inv_i;
        m2_w = m2_w + dw * (w - mean_w);
        const R dc = c - mean_cos;
        mean_cos += dc * inv_i;
        m2_cos += dc * (c - mean_cos);
    }
    const R inv_n = 1.0f / (R)n_samples;
    const uint32_t NT = 256, NP = 512;
    const R dth = (C<R>::PI * 0.5f) / (R)NT, dph = C<R>::TWO_PI / (R)NP;
    R pdf_int = 0, max_recip = 0;
    for (uint32_t ti = 0; ti < NT; ++ti) {
        const R th = ((R)ti + 0.5f) * dth;
        const R ct = std::cos(th), st = std::sin(th);
        for (uint32_t pi = 0; pi < NP; ++pi) {
            const R ph = ((R)pi + 0.5f) * dph;
            const V3<R> wo = mk(st * std::cos(ph), st * std::sin(ph), ct);
            pdf_int += pdff(wi, wo) * st * dth * dph;
            const V3<R> fio = evalf(wi, wo) / wo.z;
            const V3<R> foi = evalf(wo, wi) / wi.z;
            const R d[3] = {std::fabs(fio.x - foi.x), std::fabs(fio.y - foi.y),
                            std::fabs(fio.z - foi.z)};
            const R m[3] = {std::max(std::fabs(fio.x), std::fabs(foi.x)) + 1e-6f,
                            std::max(std::fabs(fio.y), std::fabs(foi.y)) + 1e-6f,
                            std::max(std::fabs(fio.z), std::fabs(foi.z)) + 1e-6f};
            max_recip = acc_err(max_recip, std::max(std::max(d[0] / m[0], d[1] / m[1]), d[2] / m[2]));
        }
    }
    out[0] = mean_w.x;
    out[1] = mean_w.y;
    out[2] = mean_w.z;
    out[3] = std::sqrt(m2_w.x) * inv_n;
    out[4] = std::sqrt(m2_w.y) * inv_n;
    out[5] = std::sqrt(m2_w.z) * inv_n;
    out[6] = mean_cos;
    out[7] = std::sqrt(m2_cos) * inv_n;
    out[8] = (float)valid;
    out[9] = max_w_err;
    out[10] = max_pdf_err;
    out[11] = pdf_int;
    out[12] = max_recip;
    out[13] = out[14] = out[15] = 0.0f;
    return 0;
}

// Host BVH builder: binned-SAH binary BVH, greedily collapsed to an 8-wide tree (inner children
// expanded by surface area, then free slots filled by splitting multi-triangle leaves) and written in
// the compressed-wide layout of Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on
// GPUs Through Compressed Wide BVHs" (HPG 2017): 80-byte nodes with 8-bit child boxes relative to
// a per-node origin and power-of-two scale, octant-ordered child slots, and up to three
// triangles per leaf child.
//
// merian itself hands its triangles to the Vulkan driver (BLAS/TLAS build with
// ePreferFastTrace, scene.cpp:1117-1120,1836-1882), so there is no reference builder to mirror;
// the traversal semantics that matter for parity (closest hit, culling) live in the kernels.
#include "host_common.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>

namespace gbpt {
namespace {

struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const Box& b) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow(const float* p) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    bool empty() const { return lo[0] > hi[0]; }
    float area() const {
        if (empty()) return 0.0f;
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct B2Node {
    Box box;
    uint32_t left = 0, right = 0; // children (internal)
    uint32_t first = 0, count = 0;
    bool leaf = true;
};

#ifndef GBPT_BVH_BINS
#define GBPT_BVH_BINS 32
#endif
#ifndef GBPT_BVH_TRAVERSE_COST
#define GBPT_BVH_TRAVERSE_COST 0.5f
#endif
constexpr int kMaxSplitDepth = 6;
// Split clipping halves its depth while it would make more references than this (2^28 references
// are 13 GB of triangle records and about 27 GB of host memory during the build).
constexpr size_t kMaxReferences = size_t(1) << 28;
constexpr int kBins = GBPT_BVH_BINS;
constexpr float kCostTraverse = GBPT_BVH_TRAVERSE_COST; // relative to one triangle test
constexpr uint32_t kMaxLeaf = 3;      // CWBVH leaf children hold up to three triangles
// The collapse to 8-wide nodes: SAH-optimal by dynamic programming over the binary tree (1), or
// greedy, opening the largest child until eight slots are taken (0). The DP weighs a visit of a
// wide node (its eight box tests) against one triangle test. Fitted to the closest-hit
// traversal's time on the 1M-triangle soup a triangle test costs about three node visits (lanes
// test triangles one or two at a time while node steps keep most of the warp busy); below about
// 0.7 the DP reaches the fewest triangle tests the binary leaves allow, and 0.5 measured fastest
// (1.3: 3 % slower).
#ifndef GBPT_BVH_DP_COLLAPSE
#define GBPT_BVH_DP_COLLAPSE 1
#endif
#ifndef GBPT_BVH_NODE_COST
#define GBPT_BVH_NODE_COST 0.5f
#endif
constexpr float kWideNodeCost = GBPT_BVH_NODE_COST;

struct Builder {
    const std::vector<Box>& pbox;
    const std::vector<float>& cent; // 3 per primitive
    std::vector<uint32_t>& idx;
    std::vector<B2Node> nodes;

    Builder(const std::vector<Box>& b, const std::vector<float>& c, std::vector<uint32_t>& i)
        : pbox(b), cent(c), idx(i) {}

    // Builds the subtree over idx[begin, end) into `out` (root at out[root_index]).
    void build_range(std::vector<B2Node>& out, uint32_t root_index, uint32_t begin, uint32_t end) {
        struct Task {
            uint32_t node, begin, end;
        };
        std::vector<Task> stack{{root_index, begin, end}};
        while (!stack.empty()) {
            const Task t = stack.back();
            stack.pop_back();
            const uint32_t n = t.end - t.begin;
            Box box, cbox;
            for (uint32_t i = t.begin; i < t.end; ++i) {
                box.grow(pbox[idx[i]]);
                cbox.grow(&cent[3 * idx[i]]);
            }
            out[t.node].box = box;
            out[t.node].first = t.begin;
            out[t.node].count = n;
            out[t.node].leaf = true;
            if (n <= 1) continue;

            // binned SAH over the three axes
            float best_cost = FLT_MAX;
            int best_axis = -1, best_split = 0;
            const float parent_area = std::max(box.area(), 1e-30f);
            for (int a = 0; a < 3; ++a) {
                const float ext = cbox.hi[a] - cbox.lo[a];
                if (!(ext > 0.0f)) continue;
                const float k = (float)kBins / ext;
                Box bb[kBins];
                uint32_t bn[kBins] = {};
                for (uint32_t i = t.begin; i < t.end; ++i) {
                    const uint32_t p = idx[i];
                    int b = (int)((cent[3 * p + a] - cbox.lo[a]) * k);
                    b = std::min(std::max(b, 0), kBins - 1);
                    bb[b].grow(pbox[p]);
                    bn[b]++;
                }
                float right_area[kBins];
                uint32_t right_n[kBins];
                Box acc;
                uint32_t accn = 0;
                for (int b = kBins - 1; b > 0; --b) {
                    acc.grow(bb[b]);
                    accn += bn[b];
                    right_area[b] = acc.area();
                    right_n[b] = accn;
                }
                Box lacc;
                uint32_t lacn = 0;
                for (int b = 0; b < kBins - 1; ++b) {
                    lacc.grow(bb[b]);
                    lacn += bn[b];
                    if (lacn == 0 || right_n[b + 1] == 0) continue;
                    const float c = kCostTraverse + (lacc.area() * (float)lacn +
                                                     right_area[b + 1] * (float)right_n[b + 1]) /
                                                        parent_area;
                    if (c < best_cost) {
                        best_cost = c;
                        best_axis = a;
                        best_split = b + 1;
                    }
                }
            }
            const float leaf_cost = (float)n;
            if (n <= kMaxLeaf && (best_axis < 0 || leaf_cost <= best_cost)) continue;

            uint32_t mid;
            if (best_axis < 0) {
                // all centroids coincide: split by count
                mid = t.begin + n / 2;
            } else {
                const float k = (float)kBins / (cbox.hi[best_axis] - cbox.lo[best_axis]);
                const auto it = std::partition(
                    idx.begin() + t.begin, idx.begin() + t.end, [&](uint32_t p) {
                        int b = (int)((cent[3 * p + best_axis] - cbox.lo[best_axis]) * k);
                        b = std::min(std::max(b, 0), kBins - 1);
                        return b < best_split;
                    });
                mid = (uint32_t)(it - idx.begin());
                if (mid == t.begin || mid == t.end) mid = t.begin + n / 2;
            }
            const uint32_t l = (uint32_t)out.size();
            out.emplace_back();
            out.emplace_back();
            out[t.node].leaf = false;
            out[t.node].left = l;
            out[t.node].right = l + 1;
            stack.push_back({l + 1, mid, t.end});
            stack.push_back({l, t.begin, mid});
        }
    }
};

// A fixed-capacity vector for the collapse's per-node lists (no heap traffic per node).
template <class T, int N> struct SmallVec {
    T v[N];
    size_t n = 0;
    void push_back(const T& x) { v[n++] = x; }
    size_t size() const { return n; }
    T& operator[](size_t i) { return v[i]; }
    const T& operator[](size_t i) const { return v[i]; }
    T* begin() { return v; }
    T* end() { return v + n; }
    const T* begin() const { return v; }
    const T* end() const { return v + n; }
};

// Smallest power-of-two scale with 255 * scale >= ext, as a biased exponent in [1, 254].
int quant_exponent(double ext) {
    if (!(ext > 0.0)) return 1;
    int e;
    std::frexp(ext / 255.0, &e); // ext/255 = f * 2^e, f in [0.5, 1)
    // 2^e >= ext/255 always holds; try one smaller in case ext/255 is an exact power of two
    if (std::ldexp(255.0, e - 1) >= ext) e -= 1;
    int biased = e + 127;
    return std::min(std::max(biased, 1), 254);
}

} // namespace

bool build_cwbvh(const BuildInput& in, CwBvh& out, uint32_t max_depth) {
    const size_t n = in.prim.size();
    out.nodes.clear();
    out.tris.clear();
    out.depth = 1;
    if (n == 0) {
        CwNode root{};
        root.w[3] = 127u | (127u << 8) | (127u << 16); // unit scale, no children
        out.nodes.push_back(root);
        return true;
    }
    // References: one per triangle, or several clipped pieces of a triangle whose bounding box is
    // much larger than the triangle (early split clipping, Ernst and Greiner 2007): a piece is
    // halved along its longest axis while its box area exceeds split_ratio x twice the triangle's
    // area (scaled by 1/2 per halving), at most split_depth times. Pieces keep the triangle's
    // record, so a ray may test one triangle twice; the tie rule makes that harmless.
    struct P3 {
        float x[3];
    };
    struct Piece {
        P3 poly[9]; // a triangle clipped by at most kMaxSplitDepth planes: 3 + that many corners
        int m;
        Box b;
        int depth;
    };
    static_assert(kMaxSplitDepth <= 6, "clipped pieces hold at most 9 corners");
    int split_depth = std::min(std::max(in.split_depth, 0), kMaxSplitDepth);
    const double split_ratio = std::max(in.split_ratio, 1.0);
    // references of triangles [begin, end), in triangle order
    auto make_refs = [&](size_t begin, size_t end, std::vector<Box>& boxes,
                         std::vector<uint32_t>& prims, Box& bounds) {
        std::vector<Piece> pieces;
        for (size_t i = begin; i < end; ++i) {
            const float* t = &in.v[9 * i];
            Box b;
            b.grow(t);
            b.grow(t + 3);
            b.grow(t + 6);
            bounds.grow(b);
            double area = 0.0;
            if (in.split) {
                double e1[3], e2[3];
                for (int a = 0; a < 3; ++a) {
                    e1[a] = (double)t[3 + a] - t[a];
                    e2[a] = (double)t[6 + a] - t[a];
                }
                const double cx = e1[1] * e2[2] - e1[2] * e2[1],
                             cy = e1[2] * e2[0] - e1[0] * e2[2],
                             cz = e1[0] * e2[1] - e1[1] * e2[0];
                area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
            }
            if (!(area > 0.0) || split_depth == 0 || b.area() <= split_ratio * 2.0 * area) {
                boxes.push_back(b);
                prims.push_back((uint32_t)i);
                continue;
            }
            pieces.clear();
            Piece p0;
            for (int k = 0; k < 3; ++k) std::memcpy(p0.poly[k].x, t + 3 * k, 12);
            p0.m = 3;
            p0.b = b;
            p0.depth = 0;
            pieces.push_back(p0);
            while (!pieces.empty()) {
                const Piece it = pieces.back();
                pieces.pop_back();
                if (it.depth >= split_depth ||
                    it.b.area() <= split_ratio * 2.0 * area * std::ldexp(1.0, -it.depth)) {
                    boxes.push_back(it.b);
                    prims.push_back((uint32_t)i);
                    continue;
                }
                int ax = 0;
                for (int a = 1; a < 3; ++a)
                    if (it.b.hi[a] - it.b.lo[a] > it.b.hi[ax] - it.b.lo[ax]) ax = a;
                const float mid = 0.5f * (it.b.lo[ax] + it.b.hi[ax]);
                for (int side = 0; side < 2; ++side) {
                    Piece c;
                    c.m = 0;
                    c.depth = it.depth + 1;
                    for (int k = 0; k < it.m; ++k) {
                        const P3& A = it.poly[k];
                        const P3& B = it.poly[(k + 1) % it.m];
                        const bool ina = side == 0 ? A.x[ax] <= mid : A.x[ax] >= mid;
                        const bool inb = side == 0 ? B.x[ax] <= mid : B.x[ax] >= mid;
                        if (ina) c.poly[c.m++] = A;
                        if (ina != inb) {
                            const float tt = (mid - A.x[ax]) / (B.x[ax] - A.x[ax]);
                            P3 q;
                            for (int a = 0; a < 3; ++a) q.x[a] = A.x[a] + tt * (B.x[a] - A.x[a]);
                            q.x[ax] = mid;
                            c.poly[c.m++] = q;
                        }
                    }
                    if (c.m < 3) continue;
                    for (int k = 0; k < c.m; ++k) c.b.grow(c.poly[k].x);
                    // within the parent box (rounding of the clip points)
                    for (int a = 0; a < 3; ++a) {
                        c.b.lo[a] = std::max(c.b.lo[a], it.b.lo[a]);
                        c.b.hi[a] = std::min(c.b.hi[a], it.b.hi[a]);
                    }
                    pieces.push_back(c);
                }
            }
        }
    };
    std::vector<Box> pbox;
    std::vector<uint32_t> rprim;
    Box scene;
    while (true) {
        // in parallel over contiguous triangle ranges, concatenated in order (deterministic)
        const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        const size_t parts = n < 100000 ? 1 : hw;
        std::vector<std::vector<Box>> pb(parts);
        std::vector<std::vector<uint32_t>> pp(parts);
        std::vector<Box> bounds(parts);
        std::vector<std::thread> threads;
        for (size_t k = 0; k < parts; ++k) {
            const size_t b = n * k / parts, e = n * (k + 1) / parts;
            if (parts == 1) make_refs(b, e, pb[k], pp[k], bounds[k]);
            else threads.emplace_back([&, b, e, k]() { make_refs(b, e, pb[k], pp[k], bounds[k]); });
        }
        for (auto& t : threads) t.join();
        size_t total = 0;
        for (size_t k = 0; k < parts; ++k) total += pb[k].size();
        if (total > kMaxReferences && split_depth > 0) {
            split_depth /= 2; // too many pieces: split less, at last one reference per triangle
            continue;
        }
        pbox.reserve(total);
        rprim.reserve(total);
        for (size_t k = 0; k < parts; ++k) {
            pbox.insert(pbox.end(), pb[k].begin(), pb[k].end());
            rprim.insert(rprim.end(), pp[k].begin(), pp[k].end());
            scene.grow(bounds[k]);
        }
        break;
    }
    const size_t nref = pbox.size();
    std::vector<float> cent(3 * nref);
    std::vector<uint32_t> idx(nref);
    for (size_t i = 0; i < nref; ++i) {
        for (int a = 0; a < 3; ++a) cent[3 * i + a] = 0.5f * (pbox[i].lo[a] + pbox[i].hi[a]);
        idx[i] = (uint32_t)i;
    }
    for (int a = 0; a < 3; ++a) {
        out.lo[a] = scene.lo[a];
        out.hi[a] = scene.hi[a];
    }

    Builder bld(pbox, cent, idx);
    std::vector<B2Node>& b2 = bld.nodes;
    b2.reserve(2 * nref);
    b2.emplace_back();
    // Top levels serially until there are enough independent subtrees, then the subtrees in
    // parallel into private node arrays that are appended afterwards. The partition is fixed (32
    // subtrees whatever the host's core count), so every host builds the same tree.
    {
        constexpr unsigned hw = 16;
        if (nref < 200000) {
            bld.build_range(b2, 0, 0, (uint32_t)nref);
        } else {
            // split the root range into up to 2*hw pieces by a coarse serial build (depth-limited)
            struct Part {
                uint32_t node, begin, end;
            };
            std::vector<Part> parts{{0, 0, (uint32_t)nref}};
            // expand the largest part with one SAH split at a time
            while (parts.size() < 2 * hw) {
                size_t bi = 0;
                for (size_t i = 1; i < parts.size(); ++i)
                    if (parts[i].end - parts[i].begin > parts[bi].end - parts[bi].begin) bi = i;
                const Part p = parts[bi];
                if (p.end - p.begin < 1024) break;
                {
                    Box box, cbox;
                    for (uint32_t i = p.begin; i < p.end; ++i) {
                        box.grow(pbox[idx[i]]);
                        cbox.grow(&cent[3 * idx[i]]);
                    }
                    int axis = 0;
                    for (int a = 1; a < 3; ++a)
                        if (cbox.hi[a] - cbox.lo[a] > cbox.hi[axis] - cbox.lo[axis]) axis = a;
                    // median split on the widest centroid axis keeps the parts balanced
                    const uint32_t mid = p.begin + (p.end - p.begin) / 2;
                    // ties broken by reference index: a strict order keeps the selection
                    // linear when many centroids coincide (pieces of one split triangle)
                    std::nth_element(idx.begin() + p.begin, idx.begin() + mid,
                                     idx.begin() + p.end, [&](uint32_t x, uint32_t y) {
                                         const float cx = cent[3 * x + axis], cy = cent[3 * y + axis];
                                         return cx < cy || (cx == cy && x < y);
                                     });
                    b2[p.node].box = box;
                    b2[p.node].first = p.begin;
                    b2[p.node].count = p.end - p.begin;
                    b2[p.node].leaf = false;
                    const uint32_t l = (uint32_t)b2.size();
                    b2.emplace_back();
                    b2.emplace_back();
                    b2[p.node].left = l;
                    b2[p.node].right = l + 1;
                    parts[bi] = {l, p.begin, mid};
                    parts.push_back({l + 1, mid, p.end});
                }
            }
            std::vector<std::vector<B2Node>> sub(parts.size());
            std::vector<std::thread> threads;
            for (size_t i = 0; i < parts.size(); ++i) {
                threads.emplace_back([&, i]() {
                    Builder local(pbox, cent, idx);
                    sub[i].reserve(2 * (parts[i].end - parts[i].begin));
                    sub[i].emplace_back();
                    local.build_range(sub[i], 0, parts[i].begin, parts[i].end);
                });
            }
            for (auto& t : threads) t.join();
            for (size_t i = 0; i < parts.size(); ++i) {
                const uint32_t base = (uint32_t)b2.size() - 1; // sub root replaces parts[i].node
                // sub[i][0] goes to parts[i].node; sub[i][k>0] to base + k
                auto remap = [&](uint32_t k) { return k == 0 ? parts[i].node : base + k; };
                for (size_t k = 1; k < sub[i].size(); ++k) {
                    B2Node nd = sub[i][k];
                    if (!nd.leaf) {
                        nd.left = remap(nd.left);
                        nd.right = remap(nd.right);
                    }
                    b2.push_back(nd);
                }
                B2Node root = sub[i][0];
                if (!root.leaf) {
                    root.left = remap(root.left);
                    root.right = remap(root.right);
                }
                b2[parts[i].node] = root;
            }
        }
    }

    // ---- SAH-optimal collapse (Ylitie, Karras and Laine 2017, section 3.1) -----------------
    // cost[n][i-1]: the least SAH cost of the subtree of binary node n when it fills at most i
    // child slots of a wide node (i = 1..7), in units of one triangle test; a slot holds a leaf
    // of at most three triangles or an inner child that becomes a wide node itself. choice[n]:
    // [0] 1 when n as one slot is an inner child (0: a leaf), [i-1] for i >= 2 the slots given to
    // the left child (0: the best with i - 1 slots), [7] the left child's slots when n is a wide
    // node of its own (eight slots between its two children). Children have larger indices than
    // their parents, so one pass from the back visits children first.
    bool use_dp = GBPT_BVH_DP_COLLAPSE != 0;
    std::vector<std::array<float, 7>> dp_cost;
    std::vector<std::array<uint8_t, 8>> dp_choice;
    if (use_dp) {
        dp_cost.resize(b2.size());
        dp_choice.assign(b2.size(), std::array<uint8_t, 8>{});
        for (size_t q = b2.size(); q-- > 0;) {
            const B2Node& nd = b2[q];
            const float area = nd.box.area();
            std::array<float, 7>& C = dp_cost[q];
            std::array<uint8_t, 8>& D = dp_choice[q];
            if (nd.leaf) {
                C.fill(area * (float)nd.count);
                continue;
            }
            const std::array<float, 7>& L = dp_cost[nd.left];
            const std::array<float, 7>& R = dp_cost[nd.right];
            float d8 = INFINITY;
            for (int k = 1; k <= 7; ++k) {
                const float v = L[k - 1] + R[8 - k - 1];
                if (v < d8) {
                    d8 = v;
                    D[7] = (uint8_t)k;
                }
            }
            const float as_node = area * kWideNodeCost + d8;
            const float as_leaf = nd.count <= kMaxLeaf ? area * (float)nd.count : INFINITY;
            C[0] = std::min(as_leaf, as_node);
            D[0] = as_leaf <= as_node ? 0 : 1;
            for (int i = 2; i <= 7; ++i) {
                float best = C[i - 2];
                uint8_t ch = 0;
                for (int k = 1; k < i; ++k) {
                    const float v = L[k - 1] + R[i - k - 1];
                    if (v < best) {
                        best = v;
                        ch = (uint8_t)k;
                    }
                }
                C[i - 1] = best;
                D[i - 1] = ch;
            }
        }
    }

    // ---- collapse to 8-wide and emit ----------------------------------------------------------
    struct Task {
        uint32_t b2node, cw, depth;
    };
    auto is_inner = [&](uint32_t k) { return !b2[k].leaf && b2[k].count > kMaxLeaf; };
    // the DP's children of wide node n: the slots of its two children, each slot an inner child
    // or a leaf
    auto dp_children = [&](uint32_t n, SmallVec<uint32_t, 8>& ch, bool* inner) {
        struct Item {
            uint32_t node;
            int slots;
        };
        SmallVec<Item, 16> st;
        const int k8 = dp_choice[n][7];
        st.push_back({b2[n].right, 8 - k8});
        st.push_back({b2[n].left, k8});
        while (st.size()) {
            const Item it = st.v[--st.n];
            if (it.slots == 1 || b2[it.node].leaf) {
                inner[ch.size()] = !b2[it.node].leaf && dp_choice[it.node][0] == 1;
                ch.push_back(it.node);
                continue;
            }
            const int k = dp_choice[it.node][it.slots - 1];
            if (k == 0) {
                st.push_back({it.node, it.slots - 1});
            } else {
                st.push_back({b2[it.node].right, it.slots - k});
                st.push_back({b2[it.node].left, k});
            }
        }
    };
    // One CWBVH node from task t into (nodes, tris); its inner children become tasks. Returns
    // false when the tree is deeper than max_depth.
    auto emit = [&](const Task t, std::vector<CwNode>& nodes, std::vector<TriRecord>& tris,
                    std::vector<Task>& stack, uint32_t& depth) -> bool {
        depth = std::max(depth, t.depth);
        if (t.depth > max_depth) {
            set_error("BVH deeper than the traversal stack (" + std::to_string(max_depth) + ")");
            return false;
        }
        SmallVec<uint32_t, 8> ch;
        bool inner[8] = {};
        if (use_dp && !b2[t.b2node].leaf && (t.b2node != 0 || b2[0].count > kMaxLeaf ||
                                              dp_choice[0][0] == 1)) {
            dp_children(t.b2node, ch, inner);
        } else if (is_inner(t.b2node)) {
            ch.push_back(b2[t.b2node].left);
            ch.push_back(b2[t.b2node].right);
            while (ch.size() < 8) {
                int best = -1;
                float best_area = -1.0f;
                for (size_t i = 0; i < ch.size(); ++i) {
                    if (is_inner(ch[i]) && b2[ch[i]].box.area() > best_area) {
                        best_area = b2[ch[i]].box.area();
                        best = (int)i;
                    }
                }
                if (best < 0) break;
                const uint32_t k = ch[best];
                ch[best] = b2[k].left;
                ch.push_back(b2[k].right);
            }
            // Slots left empty cost the traversal as much as full ones: split the largest
            // multi-triangle leaf children into their binary children while slots remain.
            while (ch.size() < 8) {
                int best = -1;
                float best_area = -1.0f;
                for (size_t i = 0; i < ch.size(); ++i) {
                    if (!b2[ch[i]].leaf && b2[ch[i]].box.area() > best_area) {
                        best_area = b2[ch[i]].box.area();
                        best = (int)i;
                    }
                }
                if (best < 0) break;
                const uint32_t k = ch[best];
                ch[best] = b2[k].left;
                ch.push_back(b2[k].right);
            }
            for (size_t i = 0; i < ch.size(); ++i) inner[i] = is_inner(ch[i]);
        } else {
            ch.push_back(t.b2node); // the whole tree is one leaf
        }
        // node box and centroid
        Box nbox;
        for (uint32_t c : ch) nbox.grow(b2[c].box);
        float pc[3];
        for (int a = 0; a < 3; ++a) pc[a] = 0.5f * (nbox.lo[a] + nbox.hi[a]);
        // octant slot assignment: slot s has the diagonal (+-1,+-1,+-1), sign bit a set = negative;
        // a child goes where it lies furthest back along that diagonal (first visited by rays
        // whose direction octant is s)
        const size_t m = ch.size();
        int slot_of[8];
        {
            // greedy over (child, slot) pairs in ascending (cost, child, slot) order: m rounds
            // of picking the cheapest pair whose child and slot are both free
            float cost[8][8];
            for (size_t i = 0; i < m; ++i) {
                float off[3];
                for (int a = 0; a < 3; ++a)
                    off[a] = 0.5f * (b2[ch[i]].box.lo[a] + b2[ch[i]].box.hi[a]) - pc[a];
                for (int s = 0; s < 8; ++s) {
                    float c = 0.0f;
                    for (int a = 0; a < 3; ++a) c += ((s >> a) & 1) ? -off[a] : off[a];
                    cost[i][s] = c;
                }
            }
            bool used_slot[8] = {};
            for (size_t i = 0; i < m; ++i) slot_of[i] = -1;
            for (size_t round = 0; round < m; ++round) {
                int bi = -1, bs = -1;
                for (size_t i = 0; i < m; ++i) {
                    if (slot_of[i] >= 0) continue;
                    for (int s2 = 0; s2 < 8; ++s2) {
                        if (used_slot[s2]) continue;
                        // children and slots are scanned in increasing order, so a strict
                        // comparison keeps the first (lowest child, then slot) of equal costs
                        if (bi < 0 || cost[i][s2] < cost[bi][bs]) {
                            bi = (int)i;
                            bs = s2;
                        }
                    }
                }
                slot_of[bi] = bs;
                used_slot[bs] = true;
            }
        }
        int child_at[8];
        for (int s = 0; s < 8; ++s) child_at[s] = -1;
        for (size_t i = 0; i < m; ++i) child_at[slot_of[i]] = (int)i;

        CwNode node{};
        // quantisation frame
        int ebias[3];
        for (int a = 0; a < 3; ++a) {
            const double ext = (double)nbox.hi[a] - (double)nbox.lo[a];
            ebias[a] = quant_exponent(ext);
            while (std::ldexp(255.0, ebias[a] - 127) < ext && ebias[a] < 254) ebias[a]++;
        }
        std::memcpy(&node.w[0], &nbox.lo[0], 4);
        std::memcpy(&node.w[1], &nbox.lo[1], 4);
        std::memcpy(&node.w[2], &nbox.lo[2], 4);
        uint32_t imask = 0;
        const uint32_t child_base = (uint32_t)nodes.size();
        const uint32_t tri_base = (uint32_t)tris.size();
        uint32_t n_inner = 0;
        uint8_t meta[8] = {}, qlo[3][8] = {}, qhi[3][8] = {};
        SmallVec<Task, 8> push;
        for (int s = 0; s < 8; ++s) {
            const int i = child_at[s];
            if (i < 0) continue;
            const B2Node& c = b2[ch[i]];
            for (int a = 0; a < 3; ++a) {
                const double scale = std::ldexp(1.0, ebias[a] - 127);
                double lo = std::floor(((double)c.box.lo[a] - (double)nbox.lo[a]) / scale);
                double hi = std::ceil(((double)c.box.hi[a] - (double)nbox.lo[a]) / scale);
                lo = std::min(std::max(lo, 0.0), 255.0);
                hi = std::min(std::max(hi, 0.0), 255.0);
                qlo[a][s] = (uint8_t)lo;
                qhi[a][s] = (uint8_t)hi;
            }
            if (inner[i]) {
                imask |= 1u << s;
                meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
                push.push_back({ch[i], child_base + n_inner, t.depth + 1});
                n_inner++;
            } else {
                const uint32_t off = (uint32_t)tris.size() - tri_base;
                const uint32_t cnt = c.count;
                for (uint32_t k = 0; k < cnt; ++k) {
                    const uint32_t p = rprim[idx[c.first + k]];
                    TriRecord tr{};
                    std::memcpy(tr.v0, &in.v[9 * p + 0], 12);
                    std::memcpy(tr.v1, &in.v[9 * p + 3], 12);
                    std::memcpy(tr.v2, &in.v[9 * p + 6], 12);
                    tr.prim = in.prim[p];
                    tr.geom = in.geom[p];
                    tr.pad = in.flags.empty() ? 0xFFu : in.flags[p];
                    tris.push_back(tr);
                }
                static const uint8_t unary[4] = {0, 1, 3, 7};
                meta[s] = (uint8_t)((unary[cnt] << 5) | off);
            }
        }
        node.w[3] = (uint32_t)ebias[0] | ((uint32_t)ebias[1] << 8) | ((uint32_t)ebias[2] << 16) |
                    (imask << 24);
        node.w[4] = child_base;
        node.w[5] = tri_base;
        std::memcpy(&node.w[6], meta, 8);
        std::memcpy(&node.w[8], qlo[0], 8);
        std::memcpy(&node.w[10], qlo[1], 8);
        std::memcpy(&node.w[12], qlo[2], 8);
        std::memcpy(&node.w[14], qhi[0], 8);
        std::memcpy(&node.w[16], qhi[1], 8);
        std::memcpy(&node.w[18], qhi[2], 8);
        nodes.resize(nodes.size() + n_inner);
        nodes[t.cw] = node;
        for (size_t q = push.size(); q-- > 0;) stack.push_back(push[q]);
        return true;
    };
    // The top of the tree serially until there are enough independent subtrees, then every
    // subtree into its own arrays in parallel, appended in order with rebased node and triangle
    // indices (the layout is deterministic). A DP tree deeper than max_depth falls back to the
    // greedy collapse.
    auto collapse = [&]() -> bool {
    out.nodes.clear();
    out.tris.clear();
    out.depth = 0;
    out.nodes.reserve(b2.size() / 4 + 1);
    out.tris.reserve(nref);
    out.nodes.emplace_back();
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<Task> stack{{0, 0, 1}};
    if (nref >= 200000) {
        // breadth first until the frontier holds enough subtrees (a fixed number, so the layout
        // does not depend on the host's core count)
        std::vector<Task> frontier{{0, 0, 1}};
        size_t head = 0;
        while (head < frontier.size() && frontier.size() - head < 128) {
            const Task t = frontier[head++];
            if (!emit(t, out.nodes, out.tris, frontier, out.depth)) return false;
        }
        stack.assign(frontier.begin() + (std::ptrdiff_t)head, frontier.end());
    } else {
        while (!stack.empty()) {
            const Task t = stack.back();
            stack.pop_back();
            if (!emit(t, out.nodes, out.tris, stack, out.depth)) return false;
        }
    }
    if (!stack.empty()) {
        struct Sub {
            std::vector<CwNode> nodes;
            std::vector<TriRecord> tris;
            uint32_t depth = 0;
            bool ok = true;
        };
        std::vector<Sub> subs(stack.size());
        std::vector<std::thread> threads;
        std::atomic<size_t> next{0};
        for (unsigned w = 0; w < hw; ++w) {
            threads.emplace_back([&]() {
                for (size_t i; (i = next.fetch_add(1)) < subs.size();) {
                    Sub& sb = subs[i];
                    sb.nodes.emplace_back(); // the subtree root, at local index 0
                    std::vector<Task> st{{stack[i].b2node, 0, stack[i].depth}};
                    while (!st.empty() && sb.ok) {
                        const Task t = st.back();
                        st.pop_back();
                        sb.ok = emit(t, sb.nodes, sb.tris, st, sb.depth);
                    }
                }
            });
        }
        for (auto& th : threads) th.join();
        for (size_t i = 0; i < subs.size(); ++i) {
            Sub& sb = subs[i];
            if (!sb.ok) { // the worker's message is on its own thread
                set_error("BVH deeper than the traversal stack (" + std::to_string(max_depth) + ")");
                return false;
            }
            out.depth = std::max(out.depth, sb.depth);
            // local node k >= 1 goes to base + k; the root goes to the task's reserved slot
            const uint32_t base = (uint32_t)out.nodes.size() - 1;
            const uint32_t tbase = (uint32_t)out.tris.size();
            for (size_t k = 0; k < sb.nodes.size(); ++k) {
                CwNode nd = sb.nodes[k];
                nd.w[4] += base;
                nd.w[5] += tbase;
                if (k == 0) out.nodes[stack[i].cw] = nd;
                else out.nodes.push_back(nd);
            }
            out.tris.insert(out.tris.end(), sb.tris.begin(), sb.tris.end());
        }
    }
    return true;
    };
    if (collapse()) return true;
    if (!use_dp) return false;
    use_dp = false;
    return collapse();
}

} // namespace gbpt

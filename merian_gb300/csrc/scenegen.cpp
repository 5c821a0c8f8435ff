// Seeded synthetic scenes for the benchmark configurations: a tessellated Cornell box, a
// triangle soup and a Gaussian-lobe lat-long environment. Integer PCG32 draws, one per statement,
// IEEE arithmetic without FMA contraction and the det:: transcendental functions, so a seed gives
// the same bits on every host (x86-64 and aarch64 alike).
#include "host_common.h"

#include <cmath>
#include <vector>

namespace gbpt {
namespace {

gbpt_material diffuse_material(float r, float g, float b) {
    gbpt_material m{};
    m.model = GBPT_MATERIAL_DIFFUSE;
    m.base_color[0] = r;
    m.base_color[1] = g;
    m.base_color[2] = b;
    m.specular_alpha[0] = m.specular_alpha[1] = 1.0f;
    m.specular_ior = 1.5f;
    m.base_color_texture = -1;
    return m;
}

gbpt_material openpbr_material(float r, float g, float b) {
    gbpt_material m{};
    m.model = GBPT_MATERIAL_OPENPBR;
    m.base_color[0] = r;
    m.base_color[1] = g;
    m.base_color[2] = b;
    m.metalness = 0.0f;
    m.specular_alpha[0] = m.specular_alpha[1] = 1.0f;
    m.specular_weight = 1.0f;
    m.specular_ior = 1.5f;
    m.transmission_color[0] = m.transmission_color[1] = m.transmission_color[2] = 1.0f;
    m.base_color_texture = -1;
    return m;
}

struct MeshBuilder {
    gbpt_packed_vertex* vertices;
    uint32_t* indices;
    uint32_t nv = 0, nt = 0;

    void triangle(V3 a, V3 b, V3 c) {
        const V3 n = normalize(cross(b - a, c - a));
        const uint32_t en = encode_normal(n);
        const V3 p[3] = {a, b, c};
        const float uv[3][2] = {{0.f, 0.f}, {1.f, 0.f}, {0.f, 1.f}};
        for (int k = 0; k < 3; ++k) {
            gbpt_packed_vertex& v = vertices[nv + k];
            v.position[0] = p[k].x;
            v.position[1] = p[k].y;
            v.position[2] = p[k].z;
            v.encoded_normal = en;
            v.uv = pack_half2(uv[k][0], uv[k][1]);
            v.encoded_tangent = 0;
        }
        indices[3 * nt + 0] = nv + 0;
        indices[3 * nt + 1] = nv + 1;
        indices[3 * nt + 2] = nv + 2;
        nv += 3;
        nt += 1;
    }

    // n x n grid of quads over o + [0,1]eu + [0,1]ev, front face along cross(eu, ev); cells whose
    // (i, j) satisfy pick(i, j) are emitted.
    template <class Pick, class Xf>
    void grid(V3 o, V3 eu, V3 ev, int n, Pick pick, Xf xf) {
        for (int j = 0; j < n; ++j) {
            for (int i = 0; i < n; ++i) {
                if (!pick(i, j)) continue;
                const float u0 = (float)i / n, u1 = (float)(i + 1) / n;
                const float w0 = (float)j / n, w1 = (float)(j + 1) / n;
                const V3 a = xf(o + u0 * eu + w0 * ev);
                const V3 b = xf(o + u1 * eu + w0 * ev);
                const V3 c = xf(o + u1 * eu + w1 * ev);
                const V3 d = xf(o + u0 * eu + w1 * ev);
                triangle(a, b, c);
                triangle(a, c, d);
            }
        }
    }
};

} // namespace
} // namespace gbpt

using namespace gbpt;

// The Cornell box with every grid refined `tess` times per side (1024 tess^2 triangles).
static int gen_cornell(uint64_t seed, uint32_t tess, gbpt_packed_vertex* vertices,
                       uint32_t* indices, gbpt_geometry* geometries, gbpt_material* materials) {
    if (!vertices || !indices || !geometries || !materials || tess == 0 || tess > 64) {
        set_error("gbpt_gen_cornell: null output buffer or tessellation outside [1, 64]");
        return GBPT_ERR_INVALID;
    }
    Pcg32 rng(seed, 0xC0A1u);
    float albedo[7][3];
    for (auto& a : albedo)
        for (float& c : a) c = 0.2f + 0.6f * rng.uniform();

    const int t = (int)tess, nw = 8 * t, nb = 4 * t;
    MeshBuilder mb{vertices, indices};
    const auto all = [](int, int) { return true; };
    const auto ident = [](V3 p) { return p; };
    const auto light_cell = [t](int i, int j) {
        return i >= 3 * t && i < 5 * t && j >= 3 * t && j < 5 * t;
    };
    uint32_t g = 0;
    auto begin_geom = [&](uint32_t material, uint32_t flags) {
        geometries[g].first_vertex = 0; // indices are absolute (all geometries share the pool)
        geometries[g].first_triangle = mb.nt;
        geometries[g].material_id = material;
        geometries[g].flags = flags;
        geometries[g].instance_mask = 0xFFu;
    };
    auto end_geom = [&]() {
        geometries[g].triangle_count = mb.nt - geometries[g].first_triangle;
        ++g;
    };
    // walls: front faces point into the box (counter-clockwise seen from inside)
    begin_geom(0, 0); // floor, y = 0
    mb.grid(v3(0, 0, 0), v3(0, 0, 1), v3(1, 0, 0), nw, all, ident);
    end_geom();
    begin_geom(1, 0); // ceiling without the light cells, y = 1
    mb.grid(v3(0, 1, 0), v3(1, 0, 0), v3(0, 0, 1), nw,
            [&](int i, int j) { return !light_cell(i, j); }, ident);
    end_geom();
    begin_geom(7, 0); // emissive 0.25 x 0.25 ceiling patch
    mb.grid(v3(0, 1, 0), v3(1, 0, 0), v3(0, 0, 1), nw, light_cell, ident);
    end_geom();
    begin_geom(2, 0); // back wall, z = 1
    mb.grid(v3(0, 0, 1), v3(0, 1, 0), v3(1, 0, 0), nw, all, ident);
    end_geom();
    begin_geom(3, 0); // left wall, x = 0
    mb.grid(v3(0, 0, 0), v3(0, 1, 0), v3(0, 0, 1), nw, all, ident);
    end_geom();
    begin_geom(4, 0); // right wall, x = 1
    mb.grid(v3(1, 0, 0), v3(0, 0, 1), v3(0, 1, 0), nw, all, ident);
    end_geom();

    // two boxes standing on the floor, rotated about y by -17 and +17 degrees
    const double c17 = 0.95630475596303548, s17 = 0.29237170472273677;
    struct Box {
        float sx, sy, sz, cx, cz, s;
    } boxes[2] = {{0.3f, 0.3f, 0.3f, 0.67f, 0.33f, -1.0f}, {0.3f, 0.6f, 0.3f, 0.33f, 0.67f, 1.0f}};
    for (int b = 0; b < 2; ++b) {
        const Box bx = boxes[b];
        const float cr = (float)c17, sr = (float)(bx.s * s17);
        const auto xf = [&](V3 p) {
            const float lx = (p.x - 0.5f) * bx.sx, ly = p.y * bx.sy, lz = (p.z - 0.5f) * bx.sz;
            return v3(cr * lx + sr * lz + bx.cx, ly, -sr * lx + cr * lz + bx.cz);
        };
        begin_geom(5 + b, 0);
        mb.grid(v3(1, 0, 0), v3(0, 1, 0), v3(0, 0, 1), nb, all, xf); // +x
        mb.grid(v3(0, 0, 0), v3(0, 0, 1), v3(0, 1, 0), nb, all, xf); // -x
        mb.grid(v3(0, 1, 0), v3(0, 0, 1), v3(1, 0, 0), nb, all, xf); // +y
        mb.grid(v3(0, 0, 0), v3(1, 0, 0), v3(0, 0, 1), nb, all, xf); // -y
        mb.grid(v3(0, 0, 1), v3(1, 0, 0), v3(0, 1, 0), nb, all, xf); // +z
        mb.grid(v3(0, 0, 0), v3(0, 1, 0), v3(1, 0, 0), nb, all, xf); // -z
        end_geom();
    }
    if (mb.nt != 1024u * tess * tess || g != 8) {
        set_error("gbpt_gen_cornell: internal size mismatch");
        return GBPT_ERR_INVALID;
    }
    for (int m = 0; m < 7; ++m)
        materials[m] = diffuse_material(albedo[m][0], albedo[m][1], albedo[m][2]);
    // the emitter: OpenPBR opaque dielectric with the ceiling albedo, no specular, radiance 15
    materials[7] = openpbr_material(albedo[1][0], albedo[1][1], albedo[1][2]);
    materials[7].specular_weight = 0.0f;
    materials[7].emission[0] = materials[7].emission[1] = materials[7].emission[2] = 15.0f;
    return GBPT_OK;
}

extern "C" GBPT_API int gbpt_gen_cornell(uint64_t seed, gbpt_packed_vertex* vertices,
                                         uint32_t* indices, gbpt_geometry* geometries,
                                         gbpt_material* materials) {
    return gen_cornell(seed, 1, vertices, indices, geometries, materials);
}

extern "C" GBPT_API int gbpt_gen_cornell_tess(uint64_t seed, uint32_t tess,
                                              gbpt_packed_vertex* vertices, uint32_t* indices,
                                              gbpt_geometry* geometries,
                                              gbpt_material* materials) {
    return gen_cornell(seed, tess, vertices, indices, geometries, materials);
}

extern "C" GBPT_API int gbpt_gen_soup(uint64_t seed, uint32_t n_triangles, uint32_t n_geometries,
                                      gbpt_packed_vertex* vertices, uint32_t* indices,
                                      gbpt_geometry* geometries, gbpt_material* materials) {
    if (!vertices || !indices || !geometries || !materials || n_triangles == 0 ||
        n_geometries == 0 || n_geometries > n_triangles) {
        set_error("gbpt_gen_soup: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    Pcg32 rng(seed, 0x50u);
    MeshBuilder mb{vertices, indices};
    const double mu = det::log(0.01), sigma = 0.5;
    // Marsaglia polar method: two normal deviates per accepted pair
    bool have_spare = false;
    double spare = 0.0;
    auto normal = [&]() {
        if (have_spare) {
            have_spare = false;
            return spare;
        }
        double u, v, s;
        do {
            u = 2.0 * rng.uniform_d() - 1.0;
            v = 2.0 * rng.uniform_d() - 1.0;
            s = u * u + v * v;
        } while (s >= 1.0 || s == 0.0);
        const double f = std::sqrt(-2.0 * det::log(s) / s);
        spare = v * f;
        have_spare = true;
        return u * f;
    };
    auto unit_dir = [&]() {
        float x, y, z, l2;
        do {
            x = 2.0f * rng.uniform() - 1.0f;
            y = 2.0f * rng.uniform() - 1.0f;
            z = 2.0f * rng.uniform() - 1.0f;
            l2 = x * x + y * y + z * z;
        } while (l2 > 1.0f || l2 < 1e-4f);
        const float l = std::sqrt(l2);
        return v3(x / l, y / l, z / l);
    };
    for (uint32_t g = 0; g < n_geometries; ++g) {
        const uint32_t t0 = (uint32_t)((uint64_t)n_triangles * g / n_geometries);
        const uint32_t t1 = (uint32_t)((uint64_t)n_triangles * (g + 1) / n_geometries);
        geometries[g].first_vertex = 0;
        geometries[g].first_triangle = t0;
        geometries[g].triangle_count = t1 - t0;
        geometries[g].material_id = g;
        geometries[g].flags = GBPT_MESH_TWO_SIDED | GBPT_MESH_FLAT_SHADING;
        geometries[g].instance_mask = 0xFFu;
        for (uint32_t t = t0; t < t1; ++t) {
            // one draw per statement: function-argument order is unspecified in C++ and differs
            // between compilers, which would change the scene from host to host
            const float cx = rng.uniform();
            const float cy = rng.uniform();
            const float cz = rng.uniform();
            const V3 c = v3(cx, cy, cz);
            V3 p[3];
            for (int k = 0; k < 3; ++k) {
                const float len = (float)det::exp(mu + sigma * normal());
                p[k] = c + len * unit_dir();
            }
            mb.triangle(p[0], p[1], p[2]);
        }
        const float sel = rng.uniform();
        if (sel < 0.6f) {
            const float r = 0.2f + 0.6f * rng.uniform(), gg = 0.2f + 0.6f * rng.uniform(),
                        b = 0.2f + 0.6f * rng.uniform();
            materials[g] = diffuse_material(r, gg, b);
        } else if (sel < 0.9f) {
            const float r = 0.5f + 0.5f * rng.uniform(), gg = 0.5f + 0.5f * rng.uniform(),
                        b = 0.5f + 0.5f * rng.uniform();
            const float rough = 0.05f + 0.75f * rng.uniform();
            materials[g] = openpbr_material(r, gg, b);
            materials[g].metalness = 1.0f;
            materials[g].specular_alpha[0] = materials[g].specular_alpha[1] = rough * rough;
        } else {
            const float rough = 0.05f + 0.75f * rng.uniform();
            materials[g] = openpbr_material(1.0f, 1.0f, 1.0f);
            materials[g].model = GBPT_MATERIAL_OPENPBR_TRANSMISSION;
            materials[g].specular_alpha[0] = materials[g].specular_alpha[1] = rough * rough;
            materials[g].transmission_weight = 1.0f;
        }
    }
    return GBPT_OK;
}

extern "C" GBPT_API int gbpt_gen_env(uint64_t seed, uint32_t width, uint32_t height,
                                     float* texels) {
    if (!texels || width == 0 || height == 0) {
        set_error("gbpt_gen_env: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    Pcg32 rng(seed, 0xE27u);
    struct Lobe {
        double d[3], sharp, amp[3];
    } lobes[8];
    for (Lobe& l : lobes) {
        double x, y, z, l2;
        do {
            x = 2.0 * rng.uniform_d() - 1.0;
            y = 2.0 * rng.uniform_d() - 1.0;
            z = 2.0 * rng.uniform_d() - 1.0;
            l2 = x * x + y * y + z * z;
        } while (l2 > 1.0 || l2 < 1e-4);
        const double il = 1.0 / std::sqrt(l2);
        l.d[0] = x * il;
        l.d[1] = y * il;
        l.d[2] = z * il;
        l.sharp = 5.0 + 195.0 * rng.uniform_d();
        for (double& a : l.amp) a = 0.5 + 4.5 * rng.uniform_d();
    }
    const double pi = 3.14159265358979323846;
    for (uint32_t y = 0; y < height; ++y) {
        // latlong_map_to_world (merian math.slang:254-260) at the texel centre
        const double theta = pi * ((y + 0.5) / height);
        double st, ct;
        det::sincos(theta, st, ct);
        for (uint32_t x = 0; x < width; ++x) {
            const double phi = pi * (2.0 * ((x + 0.5) / width) - 1.0);
            double sp, cp;
            det::sincos(phi, sp, cp);
            const double d[3] = {st * sp, ct, -st * cp};
            double rgb[3] = {0, 0, 0};
            for (const Lobe& l : lobes) {
                const double c = d[0] * l.d[0] + d[1] * l.d[1] + d[2] * l.d[2];
                const double w = det::exp(l.sharp * (c - 1.0));
                for (int k = 0; k < 3; ++k) rgb[k] += l.amp[k] * w;
            }
            float* t = texels + 4 * ((size_t)y * width + x);
            t[0] = (float)rgb[0];
            t[1] = (float)rgb[1];
            t[2] = (float)rgb[2];
            t[3] = 1.0f;
        }
    }
    return GBPT_OK;
}

// ---- the instanced configuration: bumpy closed meshes and value-noise textures -------------------
namespace gbpt {
namespace {

// integer lattice hash -> [0, 1)
inline float lattice(uint32_t seed, int x, int y, int z) {
    uint32_t h = seed ^ 0x9E3779B9u;
    h = (h ^ (uint32_t)x) * 0x85EBCA6Bu;
    h = (h ^ (uint32_t)y) * 0xC2B2AE35u;
    h = (h ^ (uint32_t)z) * 0x27D4EB2Fu;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}
inline float smooth(float t) { return t * t * (3.0f - 2.0f * t); }
inline float lerpf(float a, float b, float t) { return a + (b - a) * t; }

// trilinear value noise with smoothstep weights; coordinates wrap with `period` (0 = none)
float value_noise(uint32_t seed, float x, float y, float z, int period) {
    const float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const float tx = smooth(x - fx), ty = smooth(y - fy), tz = smooth(z - fz);
    auto wrap = [&](int i) { return period > 0 ? ((i % period) + period) % period : i; };
    float c[2][2][2];
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx)
                c[dz][dy][dx] = lattice(seed, wrap(ix + dx), wrap(iy + dy), wrap(iz + dz));
    const float x00 = lerpf(c[0][0][0], c[0][0][1], tx), x01 = lerpf(c[0][1][0], c[0][1][1], tx);
    const float x10 = lerpf(c[1][0][0], c[1][0][1], tx), x11 = lerpf(c[1][1][0], c[1][1][1], tx);
    return lerpf(lerpf(x00, x01, ty), lerpf(x10, x11, ty), tz);
}

} // namespace
} // namespace gbpt

// A closed bumpy sphere: an (n_u + 1) x n_v latitude-longitude vertex grid (the seam column
// duplicated for continuous uv, the pole rows collapsed), radius 1 + 0.35 * (two octaves of value
// noise - 0.5), smooth per-vertex normals (area-weighted face normals), uv = (i / n_u,
// j / (n_v - 1)); 2 n_u (n_v - 1) triangles, counter-clockwise seen from outside.
extern "C" GBPT_API int gbpt_gen_blob(uint64_t seed, uint32_t n_u, uint32_t n_v,
                                      gbpt_packed_vertex* vertices, uint32_t* indices) {
    if (!vertices || !indices || n_u < 3 || n_v < 3 || (uint64_t)(n_u + 1) * n_v > (1u << 30)) {
        set_error("gbpt_gen_blob: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    const uint32_t s32 = (uint32_t)(seed ^ (seed >> 32));
    const uint32_t nvert = (n_u + 1) * n_v;
    std::vector<V3> pos(nvert), nrm(nvert, v3(0, 0, 0));
    for (uint32_t j = 0; j < n_v; ++j) {
        const double theta = 3.14159265358979323846 * (double)j / (double)(n_v - 1);
        double st, ct;
        det::sincos(theta, st, ct);
        for (uint32_t i = 0; i <= n_u; ++i) {
            const double phi = 2.0 * 3.14159265358979323846 * (double)(i % n_u) / (double)n_u;
            double sp, cp;
            det::sincos(phi, sp, cp);
            const V3 dir = v3((float)(st * cp), (float)ct, (float)(st * sp));
            const float n1 = value_noise(s32, 2.0f * dir.x + 4.0f, 2.0f * dir.y + 4.0f, 2.0f * dir.z + 4.0f, 0);
            const float n2 = value_noise(s32 ^ 0xA5A5u, 5.0f * dir.x + 8.0f, 5.0f * dir.y + 8.0f, 5.0f * dir.z + 8.0f, 0);
            const float r = 1.0f + 0.35f * ((0.7f * n1 + 0.3f * n2) - 0.5f);
            pos[j * (n_u + 1) + i] = r * dir;
        }
    }
    uint32_t t = 0;
    for (uint32_t j = 0; j + 1 < n_v; ++j) {
        for (uint32_t i = 0; i < n_u; ++i) {
            const uint32_t a = j * (n_u + 1) + i, b = a + 1, c = a + (n_u + 1), d = c + 1;
            // (a, c, b) and (b, c, d) wind counter-clockwise seen from outside
            const uint32_t tri[2][3] = {{a, c, b}, {b, c, d}};
            for (int k = 0; k < 2; ++k) {
                indices[3 * t + 0] = tri[k][0];
                indices[3 * t + 1] = tri[k][1];
                indices[3 * t + 2] = tri[k][2];
                const V3 n = cross(pos[tri[k][1]] - pos[tri[k][0]], pos[tri[k][2]] - pos[tri[k][0]]);
                for (int q = 0; q < 3; ++q) nrm[tri[k][q]] = nrm[tri[k][q]] + n;
                ++t;
            }
        }
    }
    // the seam column shares its normals with column 0, the poles average their ring
    for (uint32_t j = 0; j < n_v; ++j) {
        V3& n0 = nrm[j * (n_u + 1)];
        V3& n1 = nrm[j * (n_u + 1) + n_u];
        const V3 s = n0 + n1;
        n0 = s;
        n1 = s;
    }
    for (uint32_t j : {0u, n_v - 1}) {
        V3 s = v3(0, 0, 0);
        for (uint32_t i = 0; i <= n_u; ++i) s = s + nrm[j * (n_u + 1) + i];
        for (uint32_t i = 0; i <= n_u; ++i) nrm[j * (n_u + 1) + i] = s;
    }
    for (uint32_t j = 0; j < n_v; ++j) {
        for (uint32_t i = 0; i <= n_u; ++i) {
            const uint32_t k = j * (n_u + 1) + i;
            gbpt_packed_vertex& v = vertices[k];
            v.position[0] = pos[k].x;
            v.position[1] = pos[k].y;
            v.position[2] = pos[k].z;
            const V3 n = dot(nrm[k], nrm[k]) > 0.0f ? normalize(nrm[k]) : normalize(pos[k]);
            v.encoded_normal = encode_normal(n);
            v.uv = pack_half2((float)i / (float)n_u, (float)j / (float)(n_v - 1));
            v.encoded_tangent = 0;
        }
    }
    return GBPT_OK;
}

// A tileable RGBA8 value-noise texture: two octaves of 2D value noise (period 8 and 16 lattice
// cells) blending two seeded colours, sRGB-encoded, alpha 255.
extern "C" GBPT_API int gbpt_gen_noise_texture(uint64_t seed, uint32_t width, uint32_t height,
                                               uint8_t* rgba) {
    if (!rgba || width == 0 || height == 0) {
        set_error("gbpt_gen_noise_texture: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    Pcg32 rng(seed, 0x7E7u);
    float c0[3], c1[3];
    for (float& c : c0) c = 0.1f + 0.8f * rng.uniform();
    for (float& c : c1) c = 0.1f + 0.8f * rng.uniform();
    const uint32_t s32 = (uint32_t)(seed ^ (seed >> 32));
    auto to_srgb8 = [](float x) {
        x = std::fmin(std::fmax(x, 0.0f), 1.0f);
        const double e = x <= 0.0031308 ? 12.92 * x : 1.055 * std::pow((double)x, 1.0 / 2.4) - 0.055;
        return (uint8_t)std::lround(e * 255.0);
    };
    for (uint32_t y = 0; y < height; ++y) {
        for (uint32_t x = 0; x < width; ++x) {
            const float u = (float)x / (float)width, v = (float)y / (float)height;
            const float n = 0.65f * value_noise(s32, 8.0f * u, 8.0f * v, 0.0f, 8) +
                            0.35f * value_noise(s32 ^ 0x5Au, 16.0f * u, 16.0f * v, 0.0f, 16);
            uint8_t* p = rgba + 4 * ((size_t)y * width + x);
            for (int c = 0; c < 3; ++c) p[c] = to_srgb8(c0[c] + (c1[c] - c0[c]) * n);
            p[3] = 255;
        }
    }
    return GBPT_OK;
}

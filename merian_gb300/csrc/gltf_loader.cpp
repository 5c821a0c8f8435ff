// glTF 2.0 scene loader (.gltf with external or data-URI buffers, and binary .glb) into the arrays
// of a gbpt_scene_desc, following what merian's GLTFScene (src/merian-shaders/scene/
// gltf_scene.cpp) reads:
//   - meshes: triangle primitives with POSITION, NORMAL, TEXCOORD_0, TANGENT and optional indices
//     (load_meshes, gltf_scene.cpp:606-700); each mesh is a BLAS, each node that holds it a TLAS
//     instance with the node's world transform (matrix, or translation x rotation x scale);
//   - mesh flags: non-OPAQUE alphaMode -> alpha-tested against the base colour texture's alpha
//     (merian: IsOpaque only for OPAQUE, alpha_texture_id = the base colour texture,
//     gltf_scene.cpp:331-334,663-675); doubleSided or KHR_materials_transmission -> TwoSided;
//     TANGENT -> HasTangents;
//   - materials, mapped onto the OpenPBR record: base colour factor x sRGB base colour texture,
//     metallic factor, GGX alpha = roughness factor^2, emissive factor x
//     KHR_materials_emissive_strength, KHR_materials_ior, KHR_materials_transmission (factor > 0:
//     the transmission model). Other textures and extensions are skipped with a warning;
//   - cameras: the first node with a perspective camera (looks down -Z, yfov, aspectRatio;
//     gltf_scene.cpp load_cameras), else a default camera looking at the scene's box.
// Images: PNG (decoded here); other formats are skipped with a warning.
#include "gbpt.h"
#include "host_common.h"
#include "json.h"
#include "loaded_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace gbpt {
namespace {

bool read_file(const std::string& path, std::vector<uint8_t>& out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    uint8_t buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + got);
    std::fclose(f);
    return true;
}

bool base64(const std::string& s, size_t from, std::vector<uint8_t>& out) {
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = from; i < s.size(); ++i) {
        const char c = s[i];
        int v;
        if (c >= 'A' && c <= 'Z') v = c - 'A';
        else if (c >= 'a' && c <= 'z') v = c - 'a' + 26;
        else if (c >= '0' && c <= '9') v = c - '0' + 52;
        else if (c == '+') v = 62;
        else if (c == '/') v = 63;
        else if (c == '=') break;
        else return false;
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)(acc >> bits));
        }
    }
    return true;
}

std::string uri_decode(const std::string& u) {
    std::string r;
    for (size_t i = 0; i < u.size(); ++i) {
        if (u[i] == '%' && i + 2 < u.size()) {
            r += (char)std::strtol(u.substr(i + 1, 2).c_str(), nullptr, 16);
            i += 2;
        } else {
            r += u[i];
        }
    }
    return r;
}

// ---- affine transforms (column-major 4x4 like glTF, double) --------------------------------
struct Mat {
    double m[16]; // column-major: m[c * 4 + r]
    static Mat identity() {
        Mat r{};
        r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0;
        return r;
    }
    double at(int r, int c) const { return m[c * 4 + r]; }
};
Mat mul(const Mat& a, const Mat& b) {
    Mat r{};
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += a.at(rr, k) * b.at(k, c);
            r.m[c * 4 + rr] = s;
        }
    return r;
}
Mat node_matrix(const Json& node) {
    if (const Json* mj = node.get("matrix"); mj && mj->size() == 16) {
        Mat r{};
        for (int i = 0; i < 16; ++i) r.m[i] = mj->a[i].n;
        return r;
    }
    double t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
    if (const Json* j = node.get("translation"); j && j->size() == 3)
        for (int i = 0; i < 3; ++i) t[i] = j->a[i].n;
    if (const Json* j = node.get("rotation"); j && j->size() == 4)
        for (int i = 0; i < 4; ++i) q[i] = j->a[i].n;
    if (const Json* j = node.get("scale"); j && j->size() == 3)
        for (int i = 0; i < 3; ++i) s[i] = j->a[i].n;
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)},
                            {2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)},
                            {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)}};
    Mat r = Mat::identity();
    for (int rr = 0; rr < 3; ++rr) {
        for (int c = 0; c < 3; ++c) r.m[c * 4 + rr] = R[rr][c] * s[c];
        r.m[12 + rr] = t[rr];
    }
    return r;
}

class Loader {
  public:
    gbpt_loaded_scene& L;
    std::string dir, err;
    Json doc;
    std::vector<std::vector<uint8_t>> buffers;
    std::vector<int> tex_map; // glTF texture -> our texture (-1: unavailable)
    std::map<std::string, bool> warned;

    explicit Loader(gbpt_loaded_scene& l) : L(l) {}

    void warn(const std::string& key, const std::string& msg) {
        if (!warned[key]) {
            warned[key] = true;
            L.warnings.push_back(msg);
        }
    }

    bool load(const std::string& path) {
        const size_t slash = path.find_last_of('/');
        dir = slash == std::string::npos ? "." : path.substr(0, slash);
        std::vector<uint8_t> file;
        if (!read_file(path, file)) return fail("cannot open " + path);
        std::vector<uint8_t> glb_bin;
        const char* js = (const char*)file.data();
        size_t jn = file.size();
        if (file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0) {
            uint32_t ver, total;
            std::memcpy(&ver, file.data() + 4, 4);
            std::memcpy(&total, file.data() + 8, 4);
            if (ver != 2 || total > file.size()) return fail("unsupported or truncated GLB");
            size_t at = 12;
            js = nullptr;
            while (at + 8 <= total) {
                uint32_t clen, ctype;
                std::memcpy(&clen, file.data() + at, 4);
                std::memcpy(&ctype, file.data() + at + 4, 4);
                if (at + 8 + (size_t)clen > total) return fail("truncated GLB chunk");
                if (ctype == 0x4E4F534Au && !js) { // JSON
                    js = (const char*)file.data() + at + 8;
                    jn = clen;
                } else if (ctype == 0x004E4942u && glb_bin.empty()) { // BIN
                    glb_bin.assign(file.data() + at + 8, file.data() + at + 8 + clen);
                }
                at += 8 + ((clen + 3) & ~3u);
            }
            if (!js) return fail("GLB without a JSON chunk");
        }
        JsonParser jp(js, js + jn);
        std::string jerr;
        if (!jp.parse(doc, jerr)) return fail(jerr);
        if (doc.type != Json::Obj) return fail("the glTF document is not a JSON object");
        if (const Json* asset = doc.get("asset")) {
            const std::string v = asset->str("version", "2.0");
            if (v.rfind("2", 0) != 0) return fail("glTF version " + v + " is not supported");
        }
        // buffers
        if (const Json* bs = doc.get("buffers")) {
            for (size_t i = 0; i < bs->size(); ++i) {
                const Json& b = bs->a[i];
                std::vector<uint8_t> data;
                const std::string uri = b.str("uri", "");
                if (uri.empty()) {
                    if (i != 0 || glb_bin.empty()) return fail("buffer without data");
                    data = glb_bin;
                } else if (uri.rfind("data:", 0) == 0) {
                    const size_t comma = uri.find(',');
                    if (comma == std::string::npos || uri.find(";base64") > comma ||
                        !base64(uri, comma + 1, data))
                        return fail("bad data URI in buffer " + std::to_string(i));
                } else if (!read_file(dir + "/" + uri_decode(uri), data)) {
                    return fail("cannot read buffer " + uri);
                }
                if (data.size() < (size_t)b.num("byteLength", 0)) return fail("buffer too short");
                buffers.push_back(std::move(data));
            }
        }
        load_textures();
        if (!load_scene()) return false;
        return true;
    }

  private:
    bool fail(const std::string& m) {
        err = m;
        return false;
    }

    // Raw bytes of a buffer view: pointer and length.
    bool view(int vi, const uint8_t*& p, size_t& n, size_t& stride) {
        const Json* views = doc.get("bufferViews");
        if (!views || vi < 0 || (size_t)vi >= views->size()) return false;
        const Json& v = views->a[vi];
        const int bi = v.idx("buffer");
        if (bi < 0 || (size_t)bi >= buffers.size()) return false;
        const size_t off = (size_t)v.num("byteOffset", 0), len = (size_t)v.num("byteLength", 0);
        if (off + len > buffers[bi].size()) return false;
        p = buffers[bi].data() + off;
        n = len;
        stride = (size_t)v.num("byteStride", 0);
        return true;
    }

    // An accessor as doubles, `comps` per element (normalized integers mapped to [0,1]/[-1,1]).
    bool accessor(int ai, int comps, std::vector<double>& out, size_t& count) {
        const Json* accs = doc.get("accessors");
        if (!accs || ai < 0 || (size_t)ai >= accs->size()) return false;
        const Json& a = accs->a[ai];
        if (a.get("sparse")) warn("sparse", "sparse accessors are not supported");
        static const std::map<std::string, int> types = {
            {"SCALAR", 1}, {"VEC2", 2}, {"VEC3", 3}, {"VEC4", 4}, {"MAT4", 16}};
        const auto ti = types.find(a.str("type", ""));
        if (ti == types.end() || ti->second != comps) return false;
        const int ct = a.idx("componentType");
        int csize;
        switch (ct) {
        case 5120: case 5121: csize = 1; break;
        case 5122: case 5123: csize = 2; break;
        case 5125: case 5126: csize = 4; break;
        default: return false;
        }
        count = (size_t)a.num("count", 0);
        out.assign(count * comps, 0.0);
        const int bv = a.idx("bufferView");
        if (bv < 0) return true; // all zeros
        const uint8_t* p;
        size_t n, stride;
        if (!view(bv, p, n, stride)) return false;
        const size_t off = (size_t)a.num("byteOffset", 0);
        const size_t elem = (size_t)csize * comps;
        if (stride == 0) stride = elem;
        if (count && off + (count - 1) * stride + elem > n) return false;
        const bool norm = a.get("normalized") && a.get("normalized")->b;
        for (size_t i = 0; i < count; ++i)
            for (int c = 0; c < comps; ++c) {
                const uint8_t* q = p + off + i * stride + (size_t)c * csize;
                double v = 0.0;
                switch (ct) {
                case 5120: v = (int8_t)q[0]; if (norm) v = std::max(v / 127.0, -1.0); break;
                case 5121: v = q[0]; if (norm) v /= 255.0; break;
                case 5122: { int16_t x; std::memcpy(&x, q, 2); v = x; if (norm) v = std::max(v / 32767.0, -1.0); break; }
                case 5123: { uint16_t x; std::memcpy(&x, q, 2); v = x; if (norm) v /= 65535.0; break; }
                case 5125: { uint32_t x; std::memcpy(&x, q, 4); v = x; break; }
                default: { float x; std::memcpy(&x, q, 4); v = x; break; }
                }
                out[i * comps + c] = v;
            }
        return true;
    }

    void load_textures() {
        const Json* texs = doc.get("textures");
        const Json* imgs = doc.get("images");
        tex_map.assign(texs ? texs->size() : 0, -1);
        std::map<int, int> by_image;
        for (size_t t = 0; texs && t < texs->size(); ++t) {
            const int src = texs->a[t].idx("source");
            if (src < 0 || !imgs || (size_t)src >= imgs->size()) {
                warn("tex_src", "a texture without a PNG source is skipped");
                continue;
            }
            auto it = by_image.find(src);
            if (it != by_image.end()) {
                tex_map[t] = it->second;
                continue;
            }
            const Json& img = imgs->a[src];
            std::vector<uint8_t> bytes;
            const std::string uri = img.str("uri", "");
            const std::string mime = img.str("mimeType", "");
            bool ok = false;
            if (!uri.empty()) {
                if (uri.rfind("data:", 0) == 0) {
                    const size_t comma = uri.find(',');
                    ok = comma != std::string::npos && base64(uri, comma + 1, bytes);
                } else {
                    ok = read_file(dir + "/" + uri_decode(uri), bytes);
                }
            } else if (img.idx("bufferView") >= 0) {
                const uint8_t* p;
                size_t n, stride;
                if ((ok = view(img.idx("bufferView"), p, n, stride))) bytes.assign(p, p + n);
            }
            std::vector<uint8_t> rgba;
            uint32_t w = 0, h = 0;
            std::string perr;
            if (!ok || !decode_png(bytes.data(), bytes.size(), rgba, w, h, perr)) {
                warn("img_" + std::to_string(src),
                     "image " + std::to_string(src) + " (" + (mime.empty() ? uri : mime) +
                         ") not loaded: " + (ok ? perr : std::string("no data")));
                continue;
            }
            const int ours = (int)L.texels.size();
            L.texels.push_back(std::move(rgba));
            gbpt_texture tx{};
            tx.width = w;
            tx.height = h;
            tx.srgb = 1; // set per use below; base colour textures are sRGB
            L.textures.push_back(tx);
            by_image[src] = ours;
            tex_map[t] = ours;
        }
        for (size_t i = 0; i < L.textures.size(); ++i) L.textures[i].texels = L.texels[i].data();
    }

    int texture_of(const Json* info) {
        if (!info) return -1;
        const int t = info->idx("index");
        if (t < 0 || (size_t)t >= tex_map.size()) return -1;
        if (info->num("texCoord", 0) != 0) warn("texcoord1", "TEXCOORD_1 textures are not supported");
        return tex_map[t];
    }

    // our material record and mesh flags for glTF material m (-1: the glTF default)
    std::pair<gbpt_material, uint32_t> material(int m) {
        gbpt_material r{};
        r.model = GBPT_MATERIAL_OPENPBR;
        r.base_color[0] = r.base_color[1] = r.base_color[2] = 1.0f;
        r.metalness = 1.0f;
        r.specular_alpha[0] = r.specular_alpha[1] = 1.0f;
        r.specular_weight = 1.0f;
        r.specular_ior = 1.5f;
        r.transmission_color[0] = r.transmission_color[1] = r.transmission_color[2] = 1.0f;
        r.base_color_texture = -1;
        r.alpha_texture = -1;
        uint32_t flags = 0;
        const Json* mats = doc.get("materials");
        if (m < 0 || !mats || (size_t)m >= mats->size()) return {r, flags};
        const Json& g = mats->a[m];
        double rough = 1.0;
        if (const Json* pbr = g.get("pbrMetallicRoughness")) {
            if (const Json* f = pbr->get("baseColorFactor"); f && f->size() == 4)
                for (int c = 0; c < 3; ++c) r.base_color[c] = (float)f->a[c].n;
            r.metalness = (float)pbr->num("metallicFactor", 1.0);
            rough = pbr->num("roughnessFactor", 1.0);
            r.base_color_texture = texture_of(pbr->get("baseColorTexture"));
            if (pbr->get("metallicRoughnessTexture"))
                warn("mr_tex", "metallic-roughness textures are not supported (factors used)");
        }
        r.specular_alpha[0] = r.specular_alpha[1] = (float)(rough * rough);
        if (const Json* e = g.get("emissiveFactor"); e && e->size() == 3)
            for (int c = 0; c < 3; ++c) r.emission[c] = (float)e->a[c].n;
        if (g.get("emissiveTexture")) warn("em_tex", "emissive textures are not supported");
        if (g.get("normalTexture")) warn("n_tex", "normal textures are not supported");
        if (g.get("occlusionTexture")) warn("o_tex", "occlusion textures are ignored");
        bool transmissive = false;
        if (const Json* ext = g.get("extensions")) {
            for (const auto& kv : ext->o) {
                if (kv.first == "KHR_materials_emissive_strength") {
                    const float k = (float)kv.second.num("emissiveStrength", 1.0);
                    for (float& c : r.emission) c *= k;
                } else if (kv.first == "KHR_materials_ior") {
                    r.specular_ior = (float)kv.second.num("ior", 1.5);
                } else if (kv.first == "KHR_materials_transmission") {
                    transmissive = true;
                    const double w = kv.second.num("transmissionFactor", 0.0);
                    if (w > 0.0) {
                        r.model = GBPT_MATERIAL_OPENPBR_TRANSMISSION;
                        r.transmission_weight = (float)w;
                    }
                } else {
                    warn("ext_" + kv.first, "material extension " + kv.first + " is ignored");
                }
            }
        }
        const std::string mode = g.str("alphaMode", "OPAQUE");
        if (mode != "OPAQUE" && r.base_color_texture >= 0) {
            flags |= GBPT_MESH_ALPHA_TEST;
            r.alpha_texture = r.base_color_texture;
            if (mode == "BLEND") warn("blend", "alphaMode BLEND is alpha-tested at 0.5");
        }
        if ((g.get("doubleSided") && g.get("doubleSided")->b) || transmissive)
            flags |= GBPT_MESH_TWO_SIDED;
        return {r, flags};
    }

    // geometries of mesh `mi` (object space); returns false on malformed data
    bool add_mesh(int mi, std::map<int, uint32_t>& mat_ids) {
        const Json& mesh = doc.get("meshes")->a[mi];
        const Json* prims = mesh.get("primitives");
        for (size_t pi = 0; prims && pi < prims->size(); ++pi) {
            const Json& pr = prims->a[pi];
            if (pr.num("mode", 4) != 4) {
                warn("mode", "non-triangle primitives are skipped");
                continue;
            }
            const Json* attrs = pr.get("attributes");
            if (!attrs || attrs->idx("POSITION") < 0) continue;
            std::vector<double> P, Nn, UV, T, I;
            size_t nv = 0, nn = 0, nuv = 0, nt = 0, ni = 0;
            if (!accessor(attrs->idx("POSITION"), 3, P, nv))
                return fail("bad POSITION accessor in mesh " + std::to_string(mi));
            const bool has_n = attrs->idx("NORMAL") >= 0 && accessor(attrs->idx("NORMAL"), 3, Nn, nn) && nn == nv;
            const bool has_uv = attrs->idx("TEXCOORD_0") >= 0 && accessor(attrs->idx("TEXCOORD_0"), 2, UV, nuv) && nuv == nv;
            const bool has_t = attrs->idx("TANGENT") >= 0 && accessor(attrs->idx("TANGENT"), 4, T, nt) && nt == nv;
            if (pr.idx("indices") >= 0) {
                if (!accessor(pr.idx("indices"), 1, I, ni))
                    return fail("bad indices accessor in mesh " + std::to_string(mi));
            } else {
                ni = nv - nv % 3;
                I.resize(ni);
                for (size_t k = 0; k < ni; ++k) I[k] = (double)k;
            }
            std::vector<uint32_t> idx;
            for (size_t k = 0; k + 2 < ni; k += 3) {
                if (I[k] >= nv || I[k + 1] >= nv || I[k + 2] >= nv)
                    return fail("index out of range in mesh " + std::to_string(mi));
                idx.insert(idx.end(), {(uint32_t)I[k], (uint32_t)I[k + 1], (uint32_t)I[k + 2]});
            }
            if (idx.empty()) continue;
            // smooth normals when absent
            if (!has_n) {
                Nn.assign(3 * nv, 0.0);
                for (size_t k = 0; k < idx.size(); k += 3) {
                    const double* a = &P[3 * idx[k]];
                    const double* b = &P[3 * idx[k + 1]];
                    const double* c = &P[3 * idx[k + 2]];
                    const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
                    const double e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
                    const double f[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                         e1[0] * e2[1] - e1[1] * e2[0]};
                    for (int q = 0; q < 3; ++q)
                        for (int c2 = 0; c2 < 3; ++c2) Nn[3 * idx[k + q] + c2] += f[c2];
                }
            }
            const int m = pr.idx("material");
            auto mit = mat_ids.find(m);
            uint32_t flags;
            if (mit == mat_ids.end()) {
                auto mf = material(m);
                L.materials.push_back(mf.first);
                mat_ids[m] = (uint32_t)L.materials.size() - 1;
                mat_flags[m] = mf.second;
                mit = mat_ids.find(m);
            }
            flags = mat_flags[m];
            if (has_t) flags |= GBPT_MESH_HAS_TANGENTS;
            gbpt_geometry g{};
            g.first_vertex = (uint32_t)L.vertices.size();
            g.first_triangle = (uint32_t)(L.indices.size() / 3);
            g.triangle_count = (uint32_t)(idx.size() / 3);
            g.material_id = mit->second;
            g.flags = flags;
            g.instance_mask = 0xFF;
            for (size_t v = 0; v < nv; ++v) {
                gbpt_packed_vertex pv{};
                for (int c = 0; c < 3; ++c) pv.position[c] = (float)P[3 * v + c];
                pv.encoded_normal = encode_normal(normalize(
                    v3((float)Nn[3 * v], (float)Nn[3 * v + 1], (float)Nn[3 * v + 2])));
                pv.uv = has_uv ? pack_half2((float)UV[2 * v], (float)UV[2 * v + 1]) : 0u;
                if (has_t)
                    pv.encoded_tangent = (encode_normal(normalize(v3((float)T[4 * v], (float)T[4 * v + 1],
                                                                     (float)T[4 * v + 2]))) &
                                          ~1u) |
                                         (T[4 * v + 3] < 0.0 ? 1u : 0u);
                L.vertices.push_back(pv);
            }
            L.indices.insert(L.indices.end(), idx.begin(), idx.end());
            L.geometries.push_back(g);
        }
        return true;
    }

    std::map<int, uint32_t> mat_flags;

    bool load_scene() {
        const Json* meshes = doc.get("meshes");
        const Json* nodes = doc.get("nodes");
        if (!meshes || !meshes->size()) return fail("no meshes");
        // every mesh one BLAS
        std::map<int, uint32_t> mat_ids;
        std::vector<int> blas_of(meshes->size(), -1);
        for (size_t mi = 0; mi < meshes->size(); ++mi) {
            const uint32_t first = (uint32_t)L.geometries.size();
            if (!add_mesh((int)mi, mat_ids)) return false;
            const uint32_t cnt = (uint32_t)L.geometries.size() - first;
            if (!cnt) continue;
            blas_of[mi] = (int)L.blas.size();
            L.blas.push_back({first, cnt});
        }
        if (L.geometries.empty()) return fail("no triangle geometry");
        // the scene's node trees
        std::vector<int> roots;
        const Json* scenes = doc.get("scenes");
        const int si = doc.idx("scene") >= 0 ? doc.idx("scene") : 0;
        if (scenes && (size_t)si < scenes->size()) {
            if (const Json* rn = scenes->a[si].get("nodes"))
                for (const Json& r : rn->a) roots.push_back((int)r.n);
        } else if (nodes) {
            // no scene: every node that is nobody's child
            std::vector<bool> child(nodes->size(), false);
            for (const Json& n : nodes->a)
                if (const Json* c = n.get("children"))
                    for (const Json& k : c->a)
                        if ((size_t)k.n < child.size()) child[(size_t)k.n] = true;
            for (size_t i = 0; i < nodes->size(); ++i)
                if (!child[i]) roots.push_back((int)i);
        }
        bool have_camera = false;
        struct Item {
            int node;
            Mat world;
            int depth;
        };
        std::vector<Item> stack;
        for (auto it = roots.rbegin(); it != roots.rend(); ++it) stack.push_back({*it, Mat::identity(), 0});
        while (!stack.empty()) {
            const Item t = stack.back();
            stack.pop_back();
            if (!nodes || t.node < 0 || (size_t)t.node >= nodes->size() || t.depth > 256)
                return fail("bad node index or cyclic node graph");
            const Json& n = nodes->a[t.node];
            const Mat w = mul(t.world, node_matrix(n));
            const int mi = n.idx("mesh");
            if (mi >= 0 && (size_t)mi < blas_of.size() && blas_of[mi] >= 0) {
                gbpt_instance in{};
                in.blas = (uint32_t)blas_of[mi];
                in.mask = 0xFF;
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 4; ++c) in.object_to_world[4 * r + c] = (float)w.at(r, c);
                L.instances.push_back(in);
            }
            if (n.get("skin") || n.get("weights")) warn("skin", "skins and morph targets are ignored");
            const int ci = n.idx("camera");
            if (ci >= 0 && !have_camera) have_camera = camera(ci, w);
            if (const Json* c = n.get("children"))
                for (auto it = c->a.rbegin(); it != c->a.rend(); ++it)
                    stack.push_back({(int)it->n, w, t.depth + 1});
        }
        if (L.instances.empty()) {
            // meshes not placed by any node: each at the identity
            for (size_t b = 0; b < L.blas.size(); ++b) {
                gbpt_instance in{};
                in.blas = (uint32_t)b;
                in.mask = 0xFF;
                in.object_to_world[0] = in.object_to_world[5] = in.object_to_world[10] = 1.0f;
                L.instances.push_back(in);
            }
            warn("no_nodes", "no node places a mesh: meshes placed at the origin");
        }
        if (!have_camera) default_camera();
        if (doc.get("extensionsUsed"))
            for (const Json& e : doc.get("extensionsUsed")->a)
                if (e.s == "KHR_lights_punctual") warn("lights", "punctual lights are not supported");
        return true;
    }

    bool camera(int ci, const Mat& w) {
        const Json* cams = doc.get("cameras");
        if (!cams || (size_t)ci >= cams->size()) return false;
        const Json& c = cams->a[ci];
        if (c.str("type", "") != "perspective" || !c.get("perspective")) {
            warn("ortho", "orthographic cameras are not supported");
            return false;
        }
        const Json& p = *c.get("perspective");
        const double yfov = p.num("yfov", 60.0 * 3.14159265358979323846 / 180.0);
        const double aspect = p.num("aspectRatio", 16.0 / 9.0);
        L.height = 720;
        L.width = (uint32_t)std::max(1.0, std::round(720.0 * aspect));
        float pos[3], tgt[3], up[3];
        double fwd[3], upd[3];
        for (int k = 0; k < 3; ++k) {
            pos[k] = (float)w.at(k, 3);
            fwd[k] = -w.at(k, 2);
            upd[k] = w.at(k, 1);
        }
        const double lf = std::sqrt(fwd[0] * fwd[0] + fwd[1] * fwd[1] + fwd[2] * fwd[2]);
        const double lu = std::sqrt(upd[0] * upd[0] + upd[1] * upd[1] + upd[2] * upd[2]);
        if (!(lf > 0) || !(lu > 0)) return false;
        for (int k = 0; k < 3; ++k) {
            tgt[k] = (float)(pos[k] + fwd[k] / lf);
            up[k] = (float)(upd[k] / lu);
        }
        gbpt_camera_look_at(pos, tgt, up, (float)yfov, (float)aspect,
                            (float)p.num("znear", 0.01), (float)p.num("zfar", 1000.0), &L.camera);
        return true;
    }

    void default_camera() {
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        for (const gbpt_instance& in : L.instances) {
            const gbpt_blas_range& b = L.blas[in.blas];
            for (uint32_t g = b.first_geometry; g < b.first_geometry + b.geometry_count; ++g) {
                const gbpt_geometry& geo = L.geometries[g];
                for (uint32_t k = 0; k < 3 * geo.triangle_count; ++k) {
                    const float* p = L.vertices[geo.first_vertex + L.indices[3 * geo.first_triangle + k]].position;
                    for (int r = 0; r < 3; ++r) {
                        const float* m = &in.object_to_world[4 * r];
                        const float x = m[0] * p[0] + m[1] * p[1] + m[2] * p[2] + m[3];
                        lo[r] = std::min(lo[r], x);
                        hi[r] = std::max(hi[r], x);
                    }
                }
            }
        }
        float tgt[3], pos[3], up[3] = {0, 1, 0}, r = 0;
        for (int k = 0; k < 3; ++k) {
            tgt[k] = 0.5f * (lo[k] + hi[k]);
            r = std::max(r, hi[k] - lo[k]);
        }
        for (int k = 0; k < 3; ++k) pos[k] = tgt[k] + 1.5f * r;
        gbpt_camera_look_at(pos, tgt, up, (float)(60.0 * 3.14159265358979323846 / 180.0),
                            (float)L.width / (float)L.height, 0.01f, 1000.0f, &L.camera);
        warn("no_camera", "no camera in the file: a default camera looks at the scene box");
    }
};

} // namespace
} // namespace gbpt

extern "C" GBPT_API int gbpt_load_gltf(const char* path, gbpt_loaded_scene** out) {
    if (!path || !out) {
        gbpt::set_error("gbpt_load_gltf: null argument");
        return GBPT_ERR_INVALID;
    }
    *out = nullptr;
    auto L = std::make_unique<gbpt_loaded_scene>();
    gbpt::Loader ld(*L);
    if (!ld.load(path)) {
        gbpt::set_error("gbpt_load_gltf: " + ld.err);
        return GBPT_ERR_INVALID;
    }
    *out = L.release();
    return GBPT_OK;
}

// pbrt-v4 scene loader: parses a pbrt-v4 scene file into the arrays of a gbpt_scene_desc, with the
// camera and film size, following merian's PBRTScene (src/merian-shaders/scene/pbrt_scene.cpp)
// for what each directive becomes:
//   - shapes: trianglemesh / loopsubdiv (P, N, uv or st, S, indices), plymesh (ASCII and binary
//     PLY, triangles and quads), sphere (64 x 32) and disk (64 slices) tessellations
//     (pbrt_scene.cpp:533-763); a shape with constant alpha 0 is dropped;
//   - materials (convert_material, pbrt_scene.cpp:365-497): diffuse and the approximated types,
//     coateddiffuse, conductor / coatedconductor (reflectance, a named metal's F0, or F0 from eta
//     and k), dielectric / thindielectric (named glasses), mix (the more probable side); roughness
//     with pbrt's remaproughness (alpha = sqrt(roughness));
//   - AreaLightSource "diffuse" L x scale becomes the shape material's emission; a two-sided
//     emitter on a one-sided material gets a reversed second sheet (pbrt_scene.cpp:86-115,
//     812-826); all other geometry is two-sided; ReverseOrientation xor a mirroring transform sets
//     FlipFacing;
//   - ObjectBegin / ObjectEnd / ObjectInstance become BLASes and TLAS instances, shapes outside
//     objects one identity-placed BLAS (build_scene, pbrt_scene.cpp:849-919);
//   - LightSource "infinite" with a constant L x scale is a uniform environment (load_env,
//     pbrt_scene.cpp:925-969); Camera "perspective" and Film become the camera (load_camera,
//     pbrt_scene.cpp:971-1009: fov on the shorter image axis, near 0.01, far 1000).
// Unsupported features (image textures, image environments, other lights and shapes, media) are
// skipped with a warning, as the reference does.
#include "gbpt.h"
#include "host_common.h"
#include "loaded_scene.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

namespace gbpt {
namespace {

// ---- 4x4 affine transforms (double, row-major, points as columns) ----------------------------
struct M4 {
    double m[4][4];
    static M4 identity() {
        M4 r{};
        for (int i = 0; i < 4; ++i) r.m[i][i] = 1.0;
        return r;
    }
};
M4 mul(const M4& a, const M4& b) {
    M4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 4; ++k) r.m[i][j] += a.m[i][k] * b.m[k][j];
    return r;
}
double det3(const M4& a) {
    return a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) -
           a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0]) +
           a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}
// Inverse of a general 4x4 matrix (Gauss-Jordan with partial pivoting); false when singular.
bool inverse(const M4& a, M4& out) {
    double w[4][8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 8; ++j) w[i][j] = j < 4 ? a.m[i][j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(w[r][c]) > std::fabs(w[p][c])) p = r;
        if (std::fabs(w[p][c]) < 1e-300) return false;
        if (p != c)
            for (int j = 0; j < 8; ++j) std::swap(w[p][j], w[c][j]);
        const double d = w[c][c];
        for (int j = 0; j < 8; ++j) w[c][j] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double f = w[r][c];
            if (f != 0.0)
                for (int j = 0; j < 8; ++j) w[r][j] -= f * w[c][j];
        }
    }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) out.m[i][j] = w[i][j + 4];
    return true;
}
M4 translate(double x, double y, double z) {
    M4 r = M4::identity();
    r.m[0][3] = x;
    r.m[1][3] = y;
    r.m[2][3] = z;
    return r;
}
M4 scale(double x, double y, double z) {
    M4 r = M4::identity();
    r.m[0][0] = x;
    r.m[1][1] = y;
    r.m[2][2] = z;
    return r;
}
// Rotation by theta degrees about an axis (right-hand rule, as pbrt's Rotate).
M4 rotate(double theta_deg, double x, double y, double z) {
    const double len = std::sqrt(x * x + y * y + z * z);
    M4 r = M4::identity();
    if (!(len > 0.0)) return r;
    x /= len;
    y /= len;
    z /= len;
    const double t = theta_deg * 3.14159265358979323846 / 180.0;
    const double s = std::sin(t), c = std::cos(t), ic = 1.0 - c;
    r.m[0][0] = x * x * ic + c;
    r.m[0][1] = x * y * ic - z * s;
    r.m[0][2] = x * z * ic + y * s;
    r.m[1][0] = x * y * ic + z * s;
    r.m[1][1] = y * y * ic + c;
    r.m[1][2] = y * z * ic - x * s;
    r.m[2][0] = x * z * ic - y * s;
    r.m[2][1] = y * z * ic + x * s;
    r.m[2][2] = z * z * ic + c;
    return r;
}
// pbrt's LookAt: the camera-from-world transform of a camera at eye looking at `look`.
M4 look_at(const double e[3], const double l[3], const double u[3]) {
    double dir[3] = {l[0] - e[0], l[1] - e[1], l[2] - e[2]};
    auto norm = [](double* v) {
        const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (n > 0)
            for (int k = 0; k < 3; ++k) v[k] /= n;
    };
    auto cross = [](const double* a, const double* b, double* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    norm(dir);
    double up[3] = {u[0], u[1], u[2]}, right[3], nup[3];
    norm(up);
    cross(up, dir, right);
    norm(right);
    cross(dir, right, nup);
    M4 wfc = M4::identity(); // world from camera: columns right, up, dir, eye
    for (int k = 0; k < 3; ++k) {
        wfc.m[k][0] = right[k];
        wfc.m[k][1] = nup[k];
        wfc.m[k][2] = dir[k];
        wfc.m[k][3] = e[k];
    }
    M4 cfw;
    if (!inverse(wfc, cfw)) return M4::identity();
    return cfw;
}

// ---- tokens and parameters --------------------------------------------------------------------
struct Token {
    enum Kind { Word, String, Number, Open, Close } kind;
    std::string text;
    double num = 0.0;
};

struct Param {
    std::string type, name;
    std::vector<double> nums;
    std::vector<std::string> strs;
};

struct Params {
    std::vector<Param> list;
    const Param* find(const std::string& name) const {
        for (const Param& p : list)
            if (p.name == name) return &p;
        return nullptr;
    }
    double num(const std::string& name, double def) const {
        const Param* p = find(name);
        return p && !p->nums.empty() ? p->nums[0] : def;
    }
    std::string str(const std::string& name, const std::string& def) const {
        const Param* p = find(name);
        return p && !p->strs.empty() ? p->strs[0] : def;
    }
    bool flag(const std::string& name, bool def) const {
        const Param* p = find(name);
        if (!p) return def;
        if (!p->strs.empty()) return p->strs[0] == "true";
        if (!p->nums.empty()) return p->nums[0] != 0.0;
        return def;
    }
};

struct AreaLight {
    float radiance[3];
    bool twosided;
};

struct MaterialDesc {
    std::string type, name;
    Params params;
};

struct ShapeDesc {
    std::string type;
    Params params;
    M4 ctm;
    int material; // index into materials, -1: pbrt's default material
    bool has_light;
    AreaLight light;
    bool reverse;
    int object; // -1: placed directly
    std::string dir; // directory of the file that declared it (plymesh paths)
};

struct ObjectDesc {
    std::string name;
    M4 begin_ctm;
    std::vector<int> shapes;
};

struct InstanceDesc {
    int object;
    M4 ctm;
};

struct State {
    M4 ctm = M4::identity();
    int material = -1;
    bool has_light = false;
    AreaLight light{{0, 0, 0}, false};
    bool reverse = false;
};

} // namespace
} // namespace gbpt

namespace gbpt {
namespace {

struct TextureDesc {
    std::string cls;
    Params params;
    std::string dir;
};

class Parser {
  public:
    std::vector<MaterialDesc> materials;
    std::map<std::string, TextureDesc> textures;
    std::map<std::string, int> named_materials;
    std::vector<ShapeDesc> shapes;
    std::vector<ObjectDesc> objects;
    std::map<std::string, int> object_index;
    std::vector<InstanceDesc> instances;
    bool has_camera = false;
    M4 world_to_camera = M4::identity();
    double fov = 90.0;
    int film_w = 1280, film_h = 720;
    bool has_env = false;
    float env_radiance[3] = {1, 1, 1};
    float env_scale = 1.0f;
    std::set<std::string> warned;
    std::vector<std::string> warnings;
    std::string error;

    void warn(const std::string& key, const std::string& msg) {
        if (warned.insert(key).second) warnings.push_back(msg);
    }

    bool parse_file(const std::string& path, int depth) {
        if (depth > 16) return fail("include depth above 16 at " + path);
        std::ifstream f(path, std::ios::binary);
        if (!f) return fail("cannot open " + path);
        std::stringstream ss;
        ss << f.rdbuf();
        const std::string dir = dirname(path);
        std::vector<Token> toks;
        if (!tokenize(ss.str(), toks)) return fail(error + " in " + path);
        size_t i = 0;
        while (i < toks.size()) {
            if (toks[i].kind != Token::Word) return fail("expected a directive, got '" +
                                                         toks[i].text + "' in " + path);
            const std::string d = toks[i++].text;
            if (!directive(d, toks, i, dir, depth)) return false;
        }
        return true;
    }

  private:
    State st;
    std::vector<State> stack;
    std::map<std::string, M4> coord_sys;
    int cur_object = -1;

    bool fail(const std::string& m) {
        if (error.empty() || error.find(m) == std::string::npos) error = m;
        return false;
    }

    static std::string dirname(const std::string& p) {
        const size_t s = p.find_last_of('/');
        return s == std::string::npos ? std::string(".") : p.substr(0, s);
    }

    bool tokenize(const std::string& s, std::vector<Token>& out) {
        size_t i = 0;
        const size_t n = s.size();
        while (i < n) {
            const char c = s[i];
            if (c == '#') {
                while (i < n && s[i] != '\n') ++i;
            } else if (std::isspace((unsigned char)c)) {
                ++i;
            } else if (c == '[') {
                out.push_back({Token::Open, "[", 0});
                ++i;
            } else if (c == ']') {
                out.push_back({Token::Close, "]", 0});
                ++i;
            } else if (c == '"') {
                const size_t e = s.find('"', i + 1);
                if (e == std::string::npos) {
                    error = "unterminated string";
                    return false;
                }
                out.push_back({Token::String, s.substr(i + 1, e - i - 1), 0});
                i = e + 1;
            } else {
                size_t e = i;
                while (e < n && !std::isspace((unsigned char)s[e]) && s[e] != '[' && s[e] != ']' &&
                       s[e] != '"' && s[e] != '#')
                    ++e;
                const std::string w = s.substr(i, e - i);
                char* end = nullptr;
                const double v = std::strtod(w.c_str(), &end);
                if (end && *end == '\0' && !w.empty())
                    out.push_back({Token::Number, w, v});
                else
                    out.push_back({Token::Word, w, 0});
                i = e;
            }
        }
        return true;
    }

    bool need_nums(const std::vector<Token>& t, size_t& i, int n, double* out) {
        // bare numbers, or one bracketed list of n numbers
        bool bracket = i < t.size() && t[i].kind == Token::Open;
        if (bracket) ++i;
        for (int k = 0; k < n; ++k) {
            if (i >= t.size() || t[i].kind != Token::Number) return fail("expected a number");
            out[k] = t[i++].num;
        }
        if (bracket) {
            if (i >= t.size() || t[i].kind != Token::Close) return fail("expected ']'");
            ++i;
        }
        return true;
    }

    bool need_string(const std::vector<Token>& t, size_t& i, std::string& out) {
        if (i >= t.size() || t[i].kind != Token::String) return fail("expected a quoted string");
        out = t[i++].text;
        return true;
    }

    bool params(const std::vector<Token>& t, size_t& i, Params& out) {
        while (i < t.size() && t[i].kind == Token::String) {
            std::istringstream decl(t[i].text);
            Param p;
            decl >> p.type >> p.name;
            if (p.name.empty()) return fail("bad parameter declaration '" + t[i].text + "'");
            ++i;
            auto value = [&](const Token& v) -> bool {
                if (v.kind == Token::Number) p.nums.push_back(v.num);
                else if (v.kind == Token::String || v.kind == Token::Word) p.strs.push_back(v.text);
                else return fail("bad parameter value");
                return true;
            };
            if (i < t.size() && t[i].kind == Token::Open) {
                ++i;
                while (i < t.size() && t[i].kind != Token::Close)
                    if (!value(t[i++])) return false;
                if (i >= t.size()) return fail("unterminated parameter list");
                ++i;
            } else if (i < t.size()) {
                if (!value(t[i++])) return false;
            }
            if (p.type == "bool")
                for (std::string& s : p.strs) s = (s == "true") ? "true" : "false";
            out.list.push_back(std::move(p));
        }
        return true;
    }

    bool rgb_of(const Param& p, float out[3]) {
        if ((p.type == "rgb" || p.type == "color") && p.nums.size() >= 3) {
            for (int k = 0; k < 3; ++k) out[k] = (float)p.nums[k];
            return true;
        }
        if (p.type == "float" && !p.nums.empty()) {
            out[0] = out[1] = out[2] = (float)p.nums[0];
            return true;
        }
        if (p.type == "spectrum" && !p.strs.empty() &&
            (p.strs[0] == "stdillum-D65" || p.strs[0] == "stdillum-D50" ||
             p.strs[0] == "stdillum-E")) {
            out[0] = out[1] = out[2] = 1.0f;
            return true;
        }
        warn("spectrum_" + p.type, "spectral parameter '" + p.name + "' of type '" + p.type +
                                       "' is not converted (default used)");
        return false;
    }

    void transform_directive(const M4& m) { st.ctm = mul(st.ctm, m); }

    bool directive(const std::string& d, const std::vector<Token>& t, size_t& i,
                   const std::string& dir, int depth) {
        double v[16];
        std::string s;
        Params p;
        if (d == "Identity") {
            st.ctm = M4::identity();
        } else if (d == "Translate") {
            if (!need_nums(t, i, 3, v)) return false;
            transform_directive(translate(v[0], v[1], v[2]));
        } else if (d == "Scale") {
            if (!need_nums(t, i, 3, v)) return false;
            transform_directive(scale(v[0], v[1], v[2]));
        } else if (d == "Rotate") {
            if (!need_nums(t, i, 4, v)) return false;
            transform_directive(rotate(v[0], v[1], v[2], v[3]));
        } else if (d == "LookAt") {
            if (!need_nums(t, i, 9, v)) return false;
            transform_directive(look_at(v, v + 3, v + 6));
        } else if (d == "Transform" || d == "ConcatTransform") {
            if (!need_nums(t, i, 16, v)) return false;
            M4 m; // the 16 values list the matrix column by column
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) m.m[r][c] = v[4 * c + r];
            if (d == "Transform") st.ctm = m;
            else transform_directive(m);
        } else if (d == "CoordinateSystem") {
            if (!need_string(t, i, s)) return false;
            coord_sys[s] = st.ctm;
        } else if (d == "CoordSysTransform") {
            if (!need_string(t, i, s)) return false;
            auto it = coord_sys.find(s);
            if (it != coord_sys.end()) st.ctm = it->second;
            else if (s == "camera" && has_camera) {
                M4 inv;
                if (inverse(world_to_camera, inv)) st.ctm = inv;
            } else warn("coordsys_" + s, "unknown coordinate system '" + s + "'");
        } else if (d == "ReverseOrientation") {
            st.reverse = !st.reverse;
        } else if (d == "AttributeBegin" || d == "TransformBegin") {
            stack.push_back(st);
        } else if (d == "AttributeEnd" || d == "TransformEnd") {
            if (stack.empty()) return fail("unmatched " + d);
            if (d == "TransformEnd") {
                st.ctm = stack.back().ctm;
            } else {
                st = stack.back();
            }
            stack.pop_back();
        } else if (d == "WorldBegin") {
            coord_sys["camera"] = M4::identity();
            if (has_camera) {
                M4 inv;
                if (inverse(world_to_camera, inv)) coord_sys["camera"] = inv;
            }
            st.ctm = M4::identity();
            coord_sys["world"] = st.ctm;
        } else if (d == "WorldEnd") {
        } else if (d == "Camera") {
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            if (s != "perspective")
                warn("camera_" + s, "camera '" + s + "' unsupported, using perspective");
            has_camera = true;
            world_to_camera = st.ctm;
            fov = p.num("fov", 90.0);
        } else if (d == "Film") {
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            film_w = (int)p.num("xresolution", 1280);
            film_h = (int)p.num("yresolution", 720);
        } else if (d == "Sampler" || d == "Integrator" || d == "PixelFilter" ||
                   d == "Accelerator" || d == "MakeNamedMedium" || d == "Attribute") {
            // settings of pbrt's own renderer (or defaults this loader does not apply)
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            if (d == "Attribute") warn("attribute", "Attribute defaults are ignored");
        } else if (d == "ColorSpace") {
            if (!need_string(t, i, s)) return false;
        } else if (d == "Option") {
            if (!params(t, i, p)) return false;
        } else if (d == "MediumInterface") {
            if (!need_string(t, i, s)) return false;
            if (i < t.size() && t[i].kind == Token::String) ++i;
            warn("media", "participating media are not supported");
        } else if (d == "Material") {
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            materials.push_back({s, "", p});
            st.material = (int)materials.size() - 1;
        } else if (d == "MakeNamedMaterial") {
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            const std::string type = p.str("type", "diffuse");
            materials.push_back({type, s, p});
            named_materials[s] = (int)materials.size() - 1;
        } else if (d == "NamedMaterial") {
            if (!need_string(t, i, s)) return false;
            auto it = named_materials.find(s);
            if (it == named_materials.end()) {
                warn("named_" + s, "unknown named material '" + s + "'");
                st.material = -1;
            } else {
                st.material = it->second;
            }
        } else if (d == "Texture") {
            std::string type, cls;
            if (!need_string(t, i, s) || !need_string(t, i, type) || !need_string(t, i, cls) ||
                !params(t, i, p))
                return false;
            textures[s] = {cls, p, dir};
        } else if (d == "AreaLightSource") {
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            if (s != "diffuse") warn("area_" + s, "area light '" + s + "' unsupported");
            AreaLight l{{1, 1, 1}, p.flag("twosided", false)};
            if (const Param* lp = p.find("L")) rgb_of(*lp, l.radiance);
            const float sc = (float)p.num("scale", 1.0);
            for (float& c : l.radiance) c *= sc;
            if (p.find("filename") || p.find("power"))
                warn("area_params", "area light 'filename'/'power' parameters are ignored");
            st.has_light = true;
            st.light = l;
        } else if (d == "LightSource") {
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            if (s != "infinite") {
                warn("light_" + s, "light source '" + s + "' unsupported");
            } else if (!p.str("filename", "").empty()) {
                warn("env_image", "image infinite lights are not supported");
            } else if (has_env) {
                warn("env_multi", "multiple infinite lights, using the first");
            } else {
                has_env = true;
                env_scale = (float)p.num("scale", 1.0);
                if (const Param* lp = p.find("L")) rgb_of(*lp, env_radiance);
            }
        } else if (d == "Shape") {
            if (!need_string(t, i, s) || !params(t, i, p)) return false;
            ShapeDesc sh{s, p, st.ctm, st.material, st.has_light, st.light, st.reverse,
                         cur_object, dir};
            shapes.push_back(std::move(sh));
            if (cur_object >= 0) objects[cur_object].shapes.push_back((int)shapes.size() - 1);
        } else if (d == "ObjectBegin") {
            if (!need_string(t, i, s)) return false;
            if (cur_object >= 0) return fail("nested ObjectBegin");
            stack.push_back(st);
            objects.push_back({s, st.ctm, {}});
            cur_object = (int)objects.size() - 1;
            object_index[s] = cur_object;
        } else if (d == "ObjectEnd") {
            if (cur_object < 0 || stack.empty()) return fail("ObjectEnd without ObjectBegin");
            cur_object = -1;
            st = stack.back();
            stack.pop_back();
        } else if (d == "ObjectInstance") {
            if (!need_string(t, i, s)) return false;
            auto it = object_index.find(s);
            if (it == object_index.end()) {
                warn("object_" + s, "unknown object '" + s + "'");
            } else {
                instances.push_back({it->second, st.ctm});
            }
        } else if (d == "Include" || d == "Import") {
            if (!need_string(t, i, s)) return false;
            const std::string path = (!s.empty() && s[0] == '/') ? s : dir + "/" + s;
            if (!parse_file(path, depth + 1)) return false;
        } else {
            return fail("unknown directive '" + d + "'");
        }
        return true;
    }
};

// ---- meshes ----------------------------------------------------------------------------------
struct Mesh {
    std::vector<float> p, n, uv, s; // 3, 3, 2, 3 per vertex (n, uv, s may be empty)
    std::vector<uint32_t> idx;
};

void smooth_normals(Mesh& m) {
    const size_t nv = m.p.size() / 3;
    std::vector<double> acc(3 * nv, 0.0);
    for (size_t t = 0; t + 2 < m.idx.size(); t += 3) {
        const uint32_t a = m.idx[t], b = m.idx[t + 1], c = m.idx[t + 2];
        double e1[3], e2[3];
        for (int k = 0; k < 3; ++k) {
            e1[k] = (double)m.p[3 * b + k] - m.p[3 * a + k];
            e2[k] = (double)m.p[3 * c + k] - m.p[3 * a + k];
        }
        const double f[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                             e1[0] * e2[1] - e1[1] * e2[0]};
        for (uint32_t v : {a, b, c})
            for (int k = 0; k < 3; ++k) acc[3 * v + k] += f[k];
    }
    m.n.assign(3 * nv, 0.0f);
    for (size_t v = 0; v < nv; ++v) {
        const double l = std::sqrt(acc[3 * v] * acc[3 * v] + acc[3 * v + 1] * acc[3 * v + 1] +
                                   acc[3 * v + 2] * acc[3 * v + 2]);
        for (int k = 0; k < 3; ++k) m.n[3 * v + k] = l > 1e-20 ? (float)(acc[3 * v + k] / l) : (k == 1);
    }
}

bool fill_trianglemesh(const Params& p, Mesh& m) {
    const Param* P = p.find("P");
    if (!P || P->nums.size() < 9) return false;
    const size_t nv = P->nums.size() / 3;
    m.p.assign(P->nums.begin(), P->nums.begin() + 3 * nv);
    if (const Param* I = p.find("indices")) {
        for (size_t k = 0; k + 2 < I->nums.size(); k += 3) {
            const double a = I->nums[k], b = I->nums[k + 1], c = I->nums[k + 2];
            if (a < 0 || b < 0 || c < 0 || a >= nv || b >= nv || c >= nv) continue;
            m.idx.insert(m.idx.end(), {(uint32_t)a, (uint32_t)b, (uint32_t)c});
        }
    } else if (nv == 3) {
        m.idx = {0, 1, 2};
    } else {
        return false;
    }
    const Param* N = p.find("N");
    if (N && N->nums.size() == 3 * nv) {
        m.n.assign(N->nums.begin(), N->nums.end());
        for (size_t v = 0; v < nv; ++v) {
            float* x = &m.n[3 * v];
            const float l = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            if (l > 1e-20f)
                for (int k = 0; k < 3; ++k) x[k] /= l;
            else
                x[0] = 0, x[1] = 1, x[2] = 0;
        }
    } else {
        smooth_normals(m);
    }
    const Param* UV = p.find("uv");
    if (!UV) UV = p.find("st");
    if (UV && UV->nums.size() == 2 * nv) m.uv.assign(UV->nums.begin(), UV->nums.end());
    const Param* S = p.find("S");
    if (S && S->nums.size() == 3 * nv) m.s.assign(S->nums.begin(), S->nums.end());
    return !m.idx.empty();
}

// PLY: "format ascii 1.0" or "binary_little_endian 1.0" (big endian is byte-swapped), a vertex
// element with x y z [nx ny nz] [u v | s t | texture_u texture_v] and a face element with a
// vertex_indices (or vertex_index) list; polygons are fanned into triangles.
bool fill_plymesh(const std::string& path, Mesh& m, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::string line;
    std::getline(f, line);
    if (line.rfind("ply", 0) != 0) {
        err = path + " is not a PLY file";
        return false;
    }
    struct Prop {
        std::string name, type, count_type; // count_type non-empty for lists
    };
    struct Elem {
        std::string name;
        size_t count;
        std::vector<Prop> props;
    };
    std::vector<Elem> elems;
    int format = 0; // 0 ascii, 1 little endian, 2 big endian
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ls(line);
        std::string kw;
        ls >> kw;
        if (kw == "format") {
            std::string fm;
            ls >> fm;
            format = fm == "ascii" ? 0 : (fm == "binary_little_endian" ? 1 : 2);
        } else if (kw == "element") {
            Elem e;
            ls >> e.name >> e.count;
            elems.push_back(e);
        } else if (kw == "property") {
            if (elems.empty()) {
                err = "PLY property before element";
                return false;
            }
            Prop pr;
            std::string t;
            ls >> t;
            if (t == "list") {
                ls >> pr.count_type >> pr.type >> pr.name;
            } else {
                pr.type = t;
                ls >> pr.name;
            }
            elems.back().props.push_back(pr);
        } else if (kw == "end_header") {
            break;
        }
    }
    auto type_size = [](const std::string& t) -> int {
        if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
        if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
        if (t == "int" || t == "uint" || t == "int32" || t == "uint32" || t == "float" ||
            t == "float32")
            return 4;
        if (t == "double" || t == "float64") return 8;
        return 0;
    };
    auto read_value = [&](const std::string& t, double& out) -> bool {
        if (format == 0) {
            f >> out;
            return (bool)f;
        }
        const int sz = type_size(t);
        if (sz == 0) return false;
        unsigned char b[8];
        if (!f.read((char*)b, sz)) return false;
        if (format == 2) std::reverse(b, b + sz);
        if (t == "char" || t == "int8") out = (double)(int8_t)b[0];
        else if (t == "uchar" || t == "uint8") out = b[0];
        else if (t == "short" || t == "int16") {
            int16_t x;
            std::memcpy(&x, b, 2);
            out = x;
        } else if (t == "ushort" || t == "uint16") {
            uint16_t x;
            std::memcpy(&x, b, 2);
            out = x;
        } else if (t == "int" || t == "int32") {
            int32_t x;
            std::memcpy(&x, b, 4);
            out = x;
        } else if (t == "uint" || t == "uint32") {
            uint32_t x;
            std::memcpy(&x, b, 4);
            out = x;
        } else if (t == "float" || t == "float32") {
            float x;
            std::memcpy(&x, b, 4);
            out = x;
        } else {
            double x;
            std::memcpy(&x, b, 8);
            out = x;
        }
        return true;
    };
    size_t nv = 0;
    for (const Elem& e : elems) {
        if (e.name == "vertex") {
            nv = e.count;
            int ix[11];
            const char* names[11] = {"x", "y", "z", "nx", "ny", "nz", "u", "v", "s", "t",
                                     "texture_u"};
            for (int k = 0; k < 11; ++k) {
                ix[k] = -1;
                for (size_t q = 0; q < e.props.size(); ++q)
                    if (e.props[q].name == names[k]) ix[k] = (int)q;
            }
            int iu = ix[6] >= 0 ? ix[6] : (ix[8] >= 0 ? ix[8] : ix[10]), iv = -1;
            for (size_t q = 0; q < e.props.size(); ++q)
                if (e.props[q].name == (ix[6] >= 0 ? "v" : (ix[8] >= 0 ? "t" : "texture_v")))
                    iv = (int)q;
            if (ix[0] < 0 || ix[1] < 0 || ix[2] < 0) {
                err = "PLY vertex without x y z";
                return false;
            }
            const bool has_n = ix[3] >= 0 && ix[4] >= 0 && ix[5] >= 0, has_uv = iu >= 0 && iv >= 0;
            m.p.resize(3 * nv);
            if (has_n) m.n.resize(3 * nv);
            if (has_uv) m.uv.resize(2 * nv);
            std::vector<double> vals(e.props.size());
            for (size_t v = 0; v < nv; ++v) {
                for (size_t q = 0; q < e.props.size(); ++q) {
                    if (!e.props[q].count_type.empty()) {
                        err = "PLY vertex list properties are not supported";
                        return false;
                    }
                    if (!read_value(e.props[q].type, vals[q])) {
                        err = "truncated PLY vertex data";
                        return false;
                    }
                }
                for (int k = 0; k < 3; ++k) m.p[3 * v + k] = (float)vals[ix[k]];
                if (has_n)
                    for (int k = 0; k < 3; ++k) m.n[3 * v + k] = (float)vals[ix[3 + k]];
                if (has_uv) {
                    m.uv[2 * v] = (float)vals[iu];
                    m.uv[2 * v + 1] = (float)vals[iv];
                }
            }
        } else if (e.name == "face") {
            for (size_t fi = 0; fi < e.count; ++fi) {
                for (const Prop& pr : e.props) {
                    if (pr.count_type.empty()) {
                        double x;
                        if (!read_value(pr.type, x)) {
                            err = "truncated PLY face data";
                            return false;
                        }
                        continue;
                    }
                    double cnt;
                    if (!read_value(pr.count_type, cnt) || cnt < 0 || cnt > 1024) {
                        err = "bad PLY face list";
                        return false;
                    }
                    std::vector<double> ids((size_t)cnt);
                    for (double& x : ids)
                        if (!read_value(pr.type, x)) {
                            err = "truncated PLY face data";
                            return false;
                        }
                    if (pr.name != "vertex_indices" && pr.name != "vertex_index") continue;
                    for (size_t k = 2; k < ids.size(); ++k) {
                        const double a = ids[0], b = ids[k - 1], c = ids[k];
                        if (a < 0 || b < 0 || c < 0 || a >= nv || b >= nv || c >= nv) continue;
                        m.idx.insert(m.idx.end(), {(uint32_t)a, (uint32_t)b, (uint32_t)c});
                    }
                }
            }
        } else {
            // skip other elements
            for (size_t k = 0; k < e.count; ++k)
                for (const Prop& pr : e.props) {
                    double x;
                    if (pr.count_type.empty()) {
                        if (!read_value(pr.type, x)) return false;
                    } else {
                        double cnt;
                        if (!read_value(pr.count_type, cnt)) return false;
                        for (int q = 0; q < (int)cnt; ++q)
                            if (!read_value(pr.type, x)) return false;
                    }
                }
        }
    }
    if (m.n.empty()) smooth_normals(m);
    else
        for (size_t v = 0; v < nv; ++v) {
            float* x = &m.n[3 * v];
            const float l = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            if (l > 1e-20f)
                for (int k = 0; k < 3; ++k) x[k] /= l;
            else
                x[0] = 0, x[1] = 1, x[2] = 0;
        }
    if (m.idx.empty()) {
        err = path + " has no triangles";
        return false;
    }
    return true;
}

void fill_sphere(const Params& p, Mesh& m) {
    const double r = p.num("radius", 1.0);
    const double zmin = std::clamp(p.num("zmin", -r), -r, r), zmax = std::clamp(p.num("zmax", r), -r, r);
    const double phimax = std::clamp(p.num("phimax", 360.0), 0.0, 360.0) * 3.14159265358979323846 / 180.0;
    const double th0 = std::acos(std::clamp(zmax / r, -1.0, 1.0));
    const double th1 = std::acos(std::clamp(zmin / r, -1.0, 1.0));
    const int S = 64, T = 32;
    for (int j = 0; j <= T; ++j) {
        const double th = th0 + (th1 - th0) * j / T;
        for (int i = 0; i <= S; ++i) {
            const double ph = phimax * i / S;
            const double n[3] = {std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th)};
            for (int k = 0; k < 3; ++k) {
                m.p.push_back((float)(r * n[k]));
                m.n.push_back((float)n[k]);
            }
            m.uv.push_back((float)i / S);
            m.uv.push_back(1.0f - (float)j / T);
        }
    }
    for (int j = 0; j < T; ++j)
        for (int i = 0; i < S; ++i) {
            const uint32_t a = j * (S + 1) + i, b = a + S + 1;
            m.idx.insert(m.idx.end(), {a, b, a + 1, a + 1, b, b + 1});
        }
}

void fill_disk(const Params& p, Mesh& m) {
    const double h = p.num("height", 0.0), r = p.num("radius", 1.0);
    const double ri = std::clamp(p.num("innerradius", 0.0), 0.0, r);
    const double phimax = std::clamp(p.num("phimax", 360.0), 0.0, 360.0) * 3.14159265358979323846 / 180.0;
    const int S = 64;
    for (int i = 0; i <= S; ++i) {
        const double ph = phimax * i / S, c = std::cos(ph), s = std::sin(ph);
        m.p.insert(m.p.end(), {(float)(r * c), (float)(r * s), (float)h, (float)(ri * c),
                               (float)(ri * s), (float)h});
        m.n.insert(m.n.end(), {0, 0, 1, 0, 0, 1});
        m.uv.insert(m.uv.end(), {(float)i / S, 0.0f, (float)i / S, 1.0f});
    }
    for (int i = 0; i < S; ++i) {
        const uint32_t a = 2 * i;
        m.idx.insert(m.idx.end(), {a, a + 2, a + 1, a + 1, a + 2, a + 3});
    }
}

// ---- materials -------------------------------------------------------------------------------
gbpt_material openpbr_default() {
    gbpt_material m{};
    m.model = GBPT_MATERIAL_OPENPBR;
    m.base_color[0] = m.base_color[1] = m.base_color[2] = 1.0f;
    m.specular_alpha[0] = m.specular_alpha[1] = 1.0f;
    m.specular_weight = 1.0f;
    m.specular_ior = 1.5f;
    m.transmission_color[0] = m.transmission_color[1] = m.transmission_color[2] = 1.0f;
    m.base_color_texture = -1;
    m.alpha_texture = -1;
    return m;
}

struct MetalF0 {
    const char* name;
    float f0[3];
};
// Linear-sRGB normal-incidence reflectance of common metals (published measured values, the same
// table merian's pbrt loader uses for pbrt's named metal spectra).
const MetalF0 kMetals[] = {{"Au", {1.000f, 0.766f, 0.336f}}, {"Ag", {0.972f, 0.960f, 0.915f}},
                           {"Al", {0.913f, 0.921f, 0.925f}}, {"Cu", {0.955f, 0.637f, 0.538f}},
                           {"Cr", {0.550f, 0.556f, 0.554f}}, {"Ni", {0.660f, 0.609f, 0.526f}},
                           {"Ti", {0.542f, 0.497f, 0.449f}}, {"W", {0.510f, 0.500f, 0.480f}}};

bool named_metal(const std::string& s, float out[3]) {
    if (s.rfind("metal-", 0) != 0) return false;
    std::string n = s.substr(6);
    if (n.size() > 4 && n.compare(n.size() - 4, 4, "-eta") == 0) n.resize(n.size() - 4);
    else if (n.size() > 2 && n.compare(n.size() - 2, 2, "-k") == 0) n.resize(n.size() - 2);
    for (const MetalF0& m : kMetals)
        if (n == m.name) {
            std::memcpy(out, m.f0, 12);
            return true;
        }
    return false;
}

class Converter {
  public:
    Parser& ps;
    gbpt_loaded_scene& L;
    std::map<std::string, std::pair<int, bool>> tex_cache; // texture name -> (index, has alpha)
    Converter(Parser& p, gbpt_loaded_scene& l) : ps(p), L(l) {}

    // An "imagemap" texture (PNG) as an RGBA8 texture of the scene: (index or -1, whether any
    // texel is not opaque); "scale" multiplies the factor.
    std::pair<int, bool> image_texture(const std::string& name, float& scale) {
        auto it = ps.textures.find(name);
        if (it == ps.textures.end()) {
            ps.warn("tex_" + name, "unknown texture '" + name + "'");
            return {-1, false};
        }
        const TextureDesc& td = it->second;
        scale = (float)td.params.num("scale", 1.0);
        if (td.cls != "imagemap") {
            ps.warn("texcls_" + td.cls, "texture class '" + td.cls + "' is not supported");
            return {-1, false};
        }
        auto c = tex_cache.find(name);
        if (c != tex_cache.end()) return c->second;
        const std::string fn = td.params.str("filename", "");
        const std::string full = (!fn.empty() && fn[0] == '/') ? fn : td.dir + "/" + fn;
        std::vector<uint8_t> rgba;
        uint32_t w = 0, h = 0;
        std::string err;
        std::pair<int, bool> r{-1, false};
        if (fn.size() < 4 || fn.compare(fn.size() - 4, 4, ".png") != 0) {
            ps.warn("img_" + fn, "image '" + fn + "' is not a PNG: not loaded");
        } else if (!read_png_file(full, rgba, w, h, err)) {
            ps.warn("img_" + fn, "image '" + fn + "' not loaded: " + err);
        } else {
            bool alpha = false;
            for (size_t k = 3; k < rgba.size(); k += 4) alpha |= rgba[k] != 255;
            gbpt_texture tx{};
            tx.width = w;
            tx.height = h;
            tx.srgb = td.params.str("encoding", "sRGB") == "linear" ? 0u : 1u;
            L.texels.push_back(std::move(rgba));
            L.textures.push_back(tx);
            r = {(int)L.textures.size() - 1, alpha};
        }
        tex_cache[name] = r;
        return r;
    }

    void roughness(const Params& p, const std::string& prefix, float alpha[2]) {
        const bool remap = p.flag("remaproughness", true);
        auto to_alpha = [remap](double r) { return (float)(remap ? std::sqrt(std::max(r, 0.0)) : r); };
        const Param* rp = p.find(prefix + "roughness");
        if (rp && rp->type == "texture")
            ps.warn("rough_tex", "roughness textures are not supported (0 used)");
        const double v = rp && !rp->nums.empty() ? rp->nums[0] : 0.0;
        alpha[0] = alpha[1] = to_alpha(v);
        const Param* u = p.find(prefix + "uroughness");
        const Param* w = p.find(prefix + "vroughness");
        if (u || w) {
            alpha[0] = to_alpha(u && !u->nums.empty() ? u->nums[0] : v);
            alpha[1] = to_alpha(w && !w->nums.empty() ? w->nums[0] : v);
        }
    }

    // A colour parameter: its value, or a texture (tex >= 0) times its scale.
    void color(const Params& p, const std::string& name, const float def[3], float out[3],
               int* tex = nullptr, bool* has_alpha = nullptr) {
        std::memcpy(out, def, 12);
        if (tex) *tex = -1;
        if (has_alpha) *has_alpha = false;
        const Param* c = p.find(name);
        if (!c) return;
        if (c->type == "texture") {
            if (c->strs.empty()) return;
            float scale = 1.0f;
            const std::pair<int, bool> t = image_texture(c->strs[0], scale);
            if (t.first >= 0 && tex) {
                out[0] = out[1] = out[2] = scale;
                *tex = t.first;
                if (has_alpha) *has_alpha = t.second;
            } else if (auto it = ps.textures.find(c->strs[0]);
                       it != ps.textures.end() && it->second.cls == "constant") {
                if (const Param* v = it->second.params.find("value")) ps_rgb(*v, out);
            }
            return;
        }
        float v[3];
        if (ps_rgb(*c, v)) std::memcpy(out, v, 12);
    }

    // reflectance with its texture: the base colour texture, and (textures with alpha) the alpha
    // test and two-sidedness merian gives such materials (pbrt_scene.cpp:380-412)
    void reflectance(const Params& p, const float def[3], gbpt_material& m, uint32_t& flags) {
        int tex = -1;
        bool alpha = false;
        color(p, "reflectance", def, m.base_color, &tex, &alpha);
        m.base_color_texture = tex;
        if (tex >= 0 && alpha) {
            m.alpha_texture = tex;
            flags |= GBPT_MESH_ALPHA_TEST | GBPT_MESH_TWO_SIDED;
        }
    }

    bool ps_rgb(const Param& c, float v[3]) {
        if ((c.type == "rgb" || c.type == "color") && c.nums.size() >= 3) {
            for (int k = 0; k < 3; ++k) v[k] = (float)c.nums[k];
            return true;
        }
        if (c.type == "float" && !c.nums.empty()) {
            v[0] = v[1] = v[2] = (float)c.nums[0];
            return true;
        }
        ps.warn("spec_" + c.name, "spectral '" + c.name + "' is not converted (default used)");
        return false;
    }

    // Returns the material and the mesh flags it needs (two-sided, alpha-tested).
    gbpt_material convert(int index, int depth, uint32_t& flags) {
        gbpt_material m = openpbr_default();
        flags = 0;
        const float half[3] = {0.5f, 0.5f, 0.5f};
        if (index < 0 || depth > 4) {
            std::memcpy(m.base_color, half, 12); // pbrt's default: coated diffuse, reflectance 0.5
            m.specular_alpha[0] = m.specular_alpha[1] = 0.0f;
            return m;
        }
        const MaterialDesc& md = ps.materials[index];
        const Params& p = md.params;
        const std::string& type = md.type;
        if (type == "diffuse" || type == "diffusetransmission" || type == "subsurface" ||
            type == "hair" || type == "measured") {
            reflectance(p, half, m, flags);
            m.specular_weight = 0.0f;
            if (type != "diffuse")
                ps.warn("mat_" + type, "material '" + type + "' approximated as diffuse");
        } else if (type == "coateddiffuse") {
            reflectance(p, half, m, flags);
            m.specular_ior = (float)p.num("eta", 1.5);
            roughness(p, "", m.specular_alpha);
        } else if (type == "conductor" || type == "coatedconductor") {
            const std::string pre = type == "coatedconductor" ? "conductor." : "";
            m.metalness = 1.0f;
            const float copper[3] = {0.955f, 0.637f, 0.538f}, r09[3] = {0.9f, 0.9f, 0.9f};
            if (p.find("reflectance")) {
                reflectance(p, r09, m, flags);
            } else {
                std::memcpy(m.base_color, copper, 12);
                const Param* eta = p.find(pre + "eta");
                const Param* k = p.find(pre + "k");
                float f0[3];
                if (eta && !eta->strs.empty() && named_metal(eta->strs[0], f0)) {
                    std::memcpy(m.base_color, f0, 12);
                } else if (eta || k) {
                    float e[3] = {0.2f, 0.2f, 0.2f}, kk[3] = {3.9f, 3.9f, 3.9f};
                    if (eta) ps_rgb(*eta, e);
                    if (k) ps_rgb(*k, kk);
                    for (int c = 0; c < 3; ++c)
                        m.base_color[c] = ((e[c] - 1) * (e[c] - 1) + kk[c] * kk[c]) /
                                          ((e[c] + 1) * (e[c] + 1) + kk[c] * kk[c]);
                }
            }
            roughness(p, pre, m.specular_alpha);
            if (type == "coatedconductor")
                ps.warn("mat_coatedconductor", "coatedconductor interface layer is ignored");
        } else if (type == "dielectric" || type == "thindielectric") {
            float eta = 1.5f;
            if (const Param* e = p.find("eta")) {
                if (!e->nums.empty()) eta = (float)e->nums[0];
                else if (!e->strs.empty() && e->strs[0] == "glass-BK7") eta = 1.5168f;
                else if (!e->strs.empty() && e->strs[0] == "glass-SF11") eta = 1.7847f;
                else ps.warn("eta_" + (e->strs.empty() ? std::string() : e->strs[0]),
                             "spectral dielectric eta is not converted (1.5 used)");
            }
            m.model = GBPT_MATERIAL_OPENPBR_TRANSMISSION;
            m.specular_ior = eta;
            m.transmission_weight = 1.0f;
            roughness(p, "", m.specular_alpha);
            flags |= GBPT_MESH_TWO_SIDED;
            if (type == "thindielectric")
                ps.warn("mat_thin", "thindielectric approximated as solid dielectric");
        } else if (type == "mix") {
            const Param* mats = p.find("materials");
            if (mats && mats->strs.size() == 2) {
                const double amount = p.num("amount", 0.5);
                const std::string& chosen = mats->strs[amount >= 0.5 ? 1 : 0];
                auto it = ps.named_materials.find(chosen);
                if (it != ps.named_materials.end()) return convert(it->second, depth + 1, flags);
                ps.warn("mix_" + chosen, "mix references unknown material '" + chosen + "'");
            }
            std::memcpy(m.base_color, half, 12);
            m.specular_weight = 0.0f;
        } else {
            ps.warn("mat_" + type, "material '" + type + "' is unsupported, using diffuse");
            std::memcpy(m.base_color, half, 12);
            m.specular_weight = 0.0f;
        }
        return m;
    }
};

void pack(const Mesh& mesh, const M4* xf, std::vector<gbpt_packed_vertex>& out) {
    const size_t nv = mesh.p.size() / 3;
    // normals by the inverse transpose of the linear part
    M4 inv_t = M4::identity();
    if (xf) {
        M4 inv;
        if (inverse(*xf, inv))
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) inv_t.m[r][c] = inv.m[c][r];
    }
    for (size_t v = 0; v < nv; ++v) {
        gbpt_packed_vertex pv{};
        const float* p = &mesh.p[3 * v];
        double n[3] = {mesh.n[3 * v], mesh.n[3 * v + 1], mesh.n[3 * v + 2]};
        double s[3] = {0, 0, 0};
        if (!mesh.s.empty())
            for (int k = 0; k < 3; ++k) s[k] = mesh.s[3 * v + k];
        if (xf) {
            double q[3], nn[3], ss[3];
            for (int r = 0; r < 3; ++r) {
                q[r] = xf->m[r][0] * p[0] + xf->m[r][1] * p[1] + xf->m[r][2] * p[2] + xf->m[r][3];
                nn[r] = inv_t.m[r][0] * n[0] + inv_t.m[r][1] * n[1] + inv_t.m[r][2] * n[2];
                ss[r] = xf->m[r][0] * s[0] + xf->m[r][1] * s[1] + xf->m[r][2] * s[2];
            }
            for (int k = 0; k < 3; ++k) {
                pv.position[k] = (float)q[k];
                n[k] = nn[k];
                s[k] = ss[k];
            }
        } else {
            for (int k = 0; k < 3; ++k) pv.position[k] = p[k];
        }
        pv.encoded_normal = encode_normal(normalize(v3((float)n[0], (float)n[1], (float)n[2])));
        pv.uv = mesh.uv.empty() ? 0u : pack_half2(mesh.uv[2 * v], mesh.uv[2 * v + 1]);
        if (!mesh.s.empty())
            pv.encoded_tangent =
                encode_normal(normalize(v3((float)s[0], (float)s[1], (float)s[2]))) & ~1u;
        out.push_back(pv);
    }
}

} // namespace
} // namespace gbpt

using namespace gbpt;

extern "C" {

GBPT_API int gbpt_load_pbrt(const char* path, gbpt_loaded_scene** out) {
    if (!path || !out) {
        set_error("gbpt_load_pbrt: null argument");
        return GBPT_ERR_INVALID;
    }
    *out = nullptr;
    Parser ps;
    if (!ps.parse_file(path, 0)) {
        set_error("gbpt_load_pbrt: " + ps.error);
        return GBPT_ERR_INVALID;
    }
    auto L = std::make_unique<gbpt_loaded_scene>();
    Converter conv(ps, *L);
    // material records per (material, emission), as merian caches them
    std::map<std::tuple<int, float, float, float>, std::pair<uint32_t, uint32_t>> cache;
    auto material_for = [&](const ShapeDesc& sh, uint32_t& mflags) -> uint32_t {
        const float* e = sh.has_light ? sh.light.radiance : nullptr;
        const auto key = std::make_tuple(sh.material, e ? e[0] : 0.f, e ? e[1] : 0.f, e ? e[2] : 0.f);
        auto it = cache.find(key);
        if (it != cache.end()) {
            mflags = it->second.second;
            return it->second.first;
        }
        gbpt_material m = conv.convert(sh.material, 0, mflags);
        if (e) std::memcpy(m.emission, e, 12);
        L->materials.push_back(m);
        const uint32_t id = (uint32_t)L->materials.size() - 1;
        cache[key] = {id, mflags};
        return id;
    };
    std::vector<int> object_use(ps.objects.size(), 0);
    for (const InstanceDesc& in : ps.instances) object_use[in.object]++;
    // one geometry per shape; xf: the transform its vertices are stored under
    auto add_shape = [&](int si, const M4* xf) -> bool {
        const ShapeDesc& sh = ps.shapes[si];
        if (const Param* a = sh.params.find("alpha")) {
            if (a->type == "texture") ps.warn("shape_alpha", "textured shape alpha is unsupported");
            else if (!a->nums.empty() && a->nums[0] == 0.0) return true;
        }
        Mesh mesh;
        if (sh.type == "trianglemesh" || sh.type == "loopsubdiv") {
            if (!fill_trianglemesh(sh.params, mesh)) {
                ps.warn("bad_mesh_" + std::to_string(si), "invalid trianglemesh skipped");
                return true;
            }
            if (sh.type == "loopsubdiv")
                ps.warn("loopsubdiv", "loading subdivision control meshes unsubdivided");
        } else if (sh.type == "plymesh") {
            const std::string fn = sh.params.str("filename", "");
            const std::string full = (!fn.empty() && fn[0] == '/') ? fn : sh.dir + "/" + fn;
            std::string err;
            if (fn.empty() || !fill_plymesh(full, mesh, err)) {
                ps.warn("ply_" + fn, "failed to load plymesh '" + fn + "': " + err);
                return true;
            }
        } else if (sh.type == "sphere") {
            fill_sphere(sh.params, mesh);
        } else if (sh.type == "disk") {
            fill_disk(sh.params, mesh);
        } else {
            ps.warn("shape_" + sh.type, "shape '" + sh.type + "' is unsupported, skipping");
            return true;
        }
        uint32_t mflags = 0;
        const uint32_t mid = material_for(sh, mflags);
        const bool two_sided_mat = (mflags & GBPT_MESH_TWO_SIDED) != 0;
        uint32_t flags = mflags & GBPT_MESH_ALPHA_TEST;
        const bool two_sided_emitter = sh.has_light && sh.light.twosided;
        if (two_sided_emitter && !two_sided_mat) {
            // a coincident reversed sheet; both stay back-face culled
            const size_t nv = mesh.p.size() / 3, nt = mesh.idx.size();
            mesh.p.insert(mesh.p.end(), mesh.p.begin(), mesh.p.begin() + 3 * nv);
            for (size_t v = 0; v < nv; ++v)
                for (int k = 0; k < 3; ++k) mesh.n.push_back(-mesh.n[3 * v + k]);
            if (!mesh.uv.empty()) mesh.uv.insert(mesh.uv.end(), mesh.uv.begin(), mesh.uv.begin() + 2 * nv);
            if (!mesh.s.empty()) mesh.s.insert(mesh.s.end(), mesh.s.begin(), mesh.s.begin() + 3 * nv);
            for (size_t t = 0; t < nt; t += 3)
                mesh.idx.insert(mesh.idx.end(), {(uint32_t)(nv + mesh.idx[t]), (uint32_t)(nv + mesh.idx[t + 2]),
                                                 (uint32_t)(nv + mesh.idx[t + 1])});
        } else {
            if (two_sided_emitter)
                ps.warn("twosided_light", "two-sided area light needs a one-sided material, "
                                          "emitting front side only");
            flags |= GBPT_MESH_TWO_SIDED;
        }
        if (sh.reverse != (det3(sh.ctm) < 0.0)) flags |= GBPT_MESH_FLIP_FACING;
        if (!mesh.s.empty()) flags |= GBPT_MESH_HAS_TANGENTS;
        gbpt_geometry g{};
        g.first_vertex = (uint32_t)L->vertices.size();
        g.first_triangle = (uint32_t)(L->indices.size() / 3);
        g.triangle_count = (uint32_t)(mesh.idx.size() / 3);
        g.material_id = mid;
        g.flags = flags;
        g.instance_mask = 0xFF;
        pack(mesh, xf, L->vertices);
        L->indices.insert(L->indices.end(), mesh.idx.begin(), mesh.idx.end());
        L->geometries.push_back(g);
        return true;
    };
    const bool two_level = !ps.instances.empty();
    // directly placed shapes (world space): one BLAS under the identity in two-level scenes
    for (size_t si = 0; si < ps.shapes.size(); ++si)
        if (ps.shapes[si].object < 0) add_shape((int)si, &ps.shapes[si].ctm);
    if (two_level) {
        const uint32_t n_world = (uint32_t)L->geometries.size();
        if (n_world) {
            L->blas.push_back({0, n_world});
            gbpt_instance in{};
            in.blas = 0;
            in.mask = 0xFF;
            in.object_to_world[0] = in.object_to_world[5] = in.object_to_world[10] = 1.0f;
            L->instances.push_back(in);
        }
        std::vector<int> blas_of(ps.objects.size(), -1);
        for (size_t oi = 0; oi < ps.objects.size(); ++oi) {
            if (!object_use[oi]) continue;
            const ObjectDesc& ob = ps.objects[oi];
            M4 inv_begin;
            if (!inverse(ob.begin_ctm, inv_begin)) inv_begin = M4::identity();
            const uint32_t first = (uint32_t)L->geometries.size();
            for (int si : ob.shapes) {
                const M4 rel = mul(inv_begin, ps.shapes[si].ctm);
                add_shape(si, &rel);
            }
            const uint32_t cnt = (uint32_t)L->geometries.size() - first;
            if (!cnt) continue;
            blas_of[oi] = (int)L->blas.size();
            L->blas.push_back({first, cnt});
        }
        for (const InstanceDesc& in : ps.instances) {
            if (blas_of[in.object] < 0) continue;
            gbpt_instance gi{};
            gi.blas = (uint32_t)blas_of[in.object];
            gi.mask = 0xFF;
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 4; ++c) gi.object_to_world[4 * r + c] = (float)in.ctm.m[r][c];
            L->instances.push_back(gi);
        }
    }
    if (L->geometries.empty()) {
        set_error("gbpt_load_pbrt: no supported geometry in " + std::string(path));
        return GBPT_ERR_INVALID;
    }
    if (L->materials.empty()) L->materials.push_back(openpbr_default());
    // environment: a uniform radiance (2 x 1 texels)
    if (ps.has_env) {
        L->has_env = true;
        L->env_texels.assign(8, 1.0f);
        for (int t = 0; t < 2; ++t)
            for (int k = 0; k < 3; ++k) L->env_texels[4 * t + k] = ps.env_radiance[k];
        L->env.texels = L->env_texels.data();
        L->env.width = 2;
        L->env.height = 1;
        L->env.to_local[0] = L->env.to_local[4] = L->env.to_local[8] = 1.0f;
        L->env.intensity = ps.env_scale;
    }
    // camera (or a default looking at the scene's box)
    L->width = (uint32_t)std::max(ps.film_w, 1);
    L->height = (uint32_t)std::max(ps.film_h, 1);
    const float aspect = (float)L->width / (float)L->height;
    float pos[3], tgt[3], up[3], fov_y;
    if (ps.has_camera) {
        M4 c2w;
        if (!inverse(ps.world_to_camera, c2w)) c2w = M4::identity();
        double fwd[3], upd[3];
        for (int k = 0; k < 3; ++k) {
            fwd[k] = c2w.m[k][2];
            upd[k] = c2w.m[k][1];
        }
        const double lf = std::sqrt(fwd[0] * fwd[0] + fwd[1] * fwd[1] + fwd[2] * fwd[2]);
        const double lu = std::sqrt(upd[0] * upd[0] + upd[1] * upd[1] + upd[2] * upd[2]);
        for (int k = 0; k < 3; ++k) {
            pos[k] = (float)c2w.m[k][3];
            tgt[k] = (float)(c2w.m[k][3] + fwd[k] / lf);
            up[k] = (float)(upd[k] / lu);
        }
        const double fov = ps.fov * 3.14159265358979323846 / 180.0;
        fov_y = (float)(L->width >= L->height ? fov : 2.0 * std::atan(std::tan(0.5 * fov) / aspect));
    } else {
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        for (const gbpt_packed_vertex& v : L->vertices)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], v.position[k]);
                hi[k] = std::max(hi[k], v.position[k]);
            }
        float r = 0;
        for (int k = 0; k < 3; ++k) {
            tgt[k] = 0.5f * (lo[k] + hi[k]);
            r = std::max(r, hi[k] - lo[k]);
        }
        for (int k = 0; k < 3; ++k) pos[k] = tgt[k] + 1.5f * r;
        up[0] = 0, up[1] = 1, up[2] = 0;
        fov_y = (float)(60.0 * 3.14159265358979323846 / 180.0);
        ps.warn("no_camera", "no camera in the file: a default camera looks at the scene box");
    }
    gbpt_camera_look_at(pos, tgt, up, fov_y, aspect, 0.01f, 1000.0f, &L->camera);
    for (size_t i = 0; i < L->textures.size(); ++i) L->textures[i].texels = L->texels[i].data();
    L->warnings = ps.warnings;
    *out = L.release();
    return GBPT_OK;
}

GBPT_API int gbpt_loaded_scene_info(const gbpt_loaded_scene* s, gbpt_loaded_info* info) {
    if (!s || !info) {
        set_error("gbpt_loaded_scene_info: null argument");
        return GBPT_ERR_INVALID;
    }
    std::memset(info, 0, sizeof(*info));
    gbpt_scene_desc& d = info->desc;
    d.vertices = s->vertices.data();
    d.vertex_count = s->vertices.size();
    d.indices = s->indices.data();
    d.triangle_count = s->indices.size() / 3;
    d.geometries = s->geometries.data();
    d.geometry_count = (uint32_t)s->geometries.size();
    d.materials = s->materials.data();
    d.material_count = (uint32_t)s->materials.size();
    d.env = s->has_env ? &s->env : nullptr;
    d.blas_ranges = s->blas.empty() ? nullptr : s->blas.data();
    d.blas_count = (uint32_t)s->blas.size();
    d.instances = s->instances.empty() ? nullptr : s->instances.data();
    d.instance_count = (uint32_t)s->instances.size();
    d.textures = s->textures.empty() ? nullptr : s->textures.data();
    d.texture_count = (uint32_t)s->textures.size();
    info->camera = s->camera;
    info->width = s->width;
    info->height = s->height;
    info->warning_count = (uint32_t)s->warnings.size();
    return GBPT_OK;
}

GBPT_API const char* gbpt_loaded_scene_warning(const gbpt_loaded_scene* s, uint32_t i) {
    if (!s || i >= s->warnings.size()) return nullptr;
    return s->warnings[i].c_str();
}

GBPT_API void gbpt_loaded_scene_free(gbpt_loaded_scene* s) { delete s; }

} // extern "C"

// merian's node graph for the nodes either side of the path tracer, hosted on libgbpt (C++).
//
// A graph JSON in merian's layout (examples/renderers/pt.json: "nodes" -> name -> {"type",
// "enabled", "properties", "outputs": ["output->node.input"]}) is loaded, its nodes are created
// by type name from a registry (src/merian-graph/graph/node_registry.cpp:60-110), connected in
// dependency order and run iteration by iteration on the context stream, as Graph::run_node calls
// Node::process (src/merian-graph/graph/graph.cpp:323-360). Each node follows merian's Node
// interface (include/merian-graph/graph/node.hpp): input and output connectors by name,
// properties by the same JSON keys and defaults, NodeStatusFlags from properties(), an error
// (merian's node_error) for a value the node cannot honour.
//
// Node types: "Render (Path-traced)" (nodes/render_pt/render_pt.cpp:94-186), "GBuffer
// (Raytraced)" (nodes/gbuffer_rt/gbuffer.cpp:33-41,155-180), "Accumulate" (nodes/accumulate/
// accumulate.cpp:150-250, static camera), "Image Write" (nodes/image_write/image_write.cpp:
// 60-380, PFM files, iteration trigger) and "Error Plot" (nodes/error_plot/error_plot.cpp:
// 63-75,245-250,320-350, the metric and its history; no split-view image).
//
// Keys a node type does not know are ignored with a warning, as merian's JSON properties read
// only the keys a node asks for. Known keys whose other values change the result in ways this
// build does not implement (a firefly filter, a frametime trigger, PNG output ...) accept their
// default only.
#include "context.h"
#include "gbpt.h"
#include "json.h"

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <new>
#include <set>
#include <stdexcept>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace gbpt {
namespace {

constexpr uint32_t kNeedsReconnect = 1u; // NodeStatusFlags (node.hpp:58-65)

struct NodeError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// A node output: texels in device memory (RGBA32F, one float, or GBuffer texels), or a small
// image on the host (Error Plot's metrics).
struct Buffer {
    void* dev = nullptr;
    std::vector<float> host;
    bool on_host = false;
    uint32_t width = 0, height = 0;
    uint32_t floats = 4; // floats per texel
    // a scene node's "scene" output: the resident scene and its camera
    bool is_scene = false;
    uint32_t scene = 0;
    gbpt_camera camera{};
    Buffer() = default;
    Buffer(const Buffer&) = delete;
    Buffer& operator=(const Buffer&) = delete;
    ~Buffer() { release(); }
    uint64_t texels() const { return (uint64_t)width * height; }
    void release() {
        if (dev) cudaFree(dev);
        dev = nullptr;
    }
    void allocate(uint32_t w, uint32_t h, uint32_t fl) {
        if (dev && w == width && h == height && fl == floats) return;
        release();
        width = w;
        height = h;
        floats = fl;
        const size_t bytes = (size_t)w * h * fl * sizeof(float);
        if (bytes && device_malloc(&dev, bytes) != cudaSuccess) {
            dev = nullptr;
            throw std::bad_alloc();
        }
        if (bytes) cudaMemset(dev, 0, bytes);
    }
};

void check_rc(int rc) {
    if (rc != GBPT_OK) throw NodeError(gbpt_last_error());
}

// ---- properties ------------------------------------------------------------------------------
struct Prop {
    enum Kind { Bool, Int, Float, Text, Options } kind;
    std::string key;
    Json value;
    std::vector<std::string> options;
    bool reconnect = false;
};

Json jbool(bool b) {
    Json j;
    j.type = Json::Bool;
    j.b = b;
    return j;
}
Json jnum(double n) {
    Json j;
    j.type = Json::Num;
    j.n = n;
    return j;
}
Json jstr(const std::string& s) {
    Json j;
    j.type = Json::Str;
    j.s = s;
    return j;
}

class Node {
  public:
    explicit Node(std::string type) : type_(std::move(type)) {}
    virtual ~Node() = default;
    const std::string& type() const { return type_; }
    virtual std::vector<std::string> inputs() const = 0;
    virtual std::vector<std::string> outputs() const = 0;

    // Sets the properties of a JSON object (nested objects: a property group such as Image
    // Write's "advanced"). Every value is checked before any is applied. Returns NeedsReconnect
    // when a connector layout changes; unknown keys go to `warnings`.
    uint32_t set_properties(const Json& obj, std::vector<std::string>& warnings,
                            const std::string& prefix = "") {
        if (obj.type != Json::Obj) throw NodeError(type_ + ": properties must be a JSON object");
        std::vector<std::pair<Prop*, const Json*>> todo;
        collect(obj, prefix, warnings, todo);
        static const Json kInf = jnum(INFINITY);
        for (auto& t : todo) // JSON has no infinity: null reads as +inf for a number property
            if (t.first->kind == Prop::Float && t.second->type == Json::Null) t.second = &kInf;
        for (auto& t : todo) {
            check_type(*t.first, *t.second);
            validate(t.first->key, *t.second);
        }
        uint32_t flags = 0;
        for (auto& t : todo) {
            Prop& p = *t.first;
            const bool changed = !same(p.value, *t.second);
            p.value = *t.second;
            if (changed && p.reconnect) flags |= kNeedsReconnect;
            flags |= on_set(p.key, changed);
        }
        return flags;
    }
    const Prop* prop(const std::string& key) const {
        for (const auto& p : props_)
            if (p.key == key) return &p;
        return nullptr;
    }
    Json all_properties() const {
        Json o;
        o.type = Json::Obj;
        for (const auto& p : props_) {
            const size_t slash = p.key.find('/');
            if (slash == std::string::npos) {
                o.o.emplace_back(p.key, p.value);
                continue;
            }
            const std::string group = p.key.substr(0, slash);
            Json* g = nullptr;
            for (auto& kv : o.o)
                if (kv.first == group) g = &kv.second;
            if (!g) {
                o.o.emplace_back(group, Json());
                g = &o.o.back().second;
                g->type = Json::Obj;
            }
            g->o.emplace_back(p.key.substr(slash + 1), p.value);
        }
        return o;
    }

    // describe_outputs: sizes the outputs from the connected inputs (nullptr: not connected) and
    // the graph's extent for nodes without an image input.
    virtual void connect(gbpt_ctx* ctx, const std::map<std::string, const Buffer*>& in,
                         uint32_t width, uint32_t height, std::vector<std::string>& warnings) = 0;
    virtual void process(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera,
                         uint64_t run_iteration, const std::map<std::string, const Buffer*>& in,
                         std::vector<std::string>& warnings) = 0;
    Buffer* output(const std::string& name) {
        auto it = outs_.find(name);
        return it == outs_.end() ? nullptr : it->second.get();
    }
    // Checkpoint of what the node carries from one iteration to the next: counters in the
    // returned JSON, images as files `base` + suffix. load_state takes them back before the next
    // connect.
    virtual Json save_state(gbpt_ctx*, const std::string&) { return Json(); }
    virtual void load_state(const Json&, const std::string&) {}

  protected:
    void add(Prop::Kind k, const std::string& key, Json def, std::vector<std::string> opts = {},
             bool reconnect = false) {
        props_.push_back(Prop{k, key, std::move(def), std::move(opts), reconnect});
    }
    void add_mask() {
        for (int b = 0; b < 8; ++b) add(Prop::Bool, std::to_string(b), jbool(true));
    }
    bool b(const std::string& k) const { return prop(k)->value.b; }
    double f(const std::string& k) const { return prop(k)->value.n; }
    int64_t i(const std::string& k) const { return (int64_t)prop(k)->value.n; }
    const std::string& s(const std::string& k) const { return prop(k)->value.s; }
    uint32_t mask() const {
        uint32_t m = 0;
        for (int bit = 0; bit < 8; ++bit)
            if (b(std::to_string(bit))) m |= 1u << bit;
        return m;
    }
    void set(const std::string& k, Json v) {
        for (auto& p : props_)
            if (p.key == k) p.value = std::move(v);
    }
    Buffer& out(const std::string& name) {
        auto& p = outs_[name];
        if (!p) p.reset(new Buffer());
        return *p;
    }
    // node-specific checks of one new value (throw NodeError), and what a set value triggers
    virtual void validate(const std::string&, const Json&) {}
    virtual uint32_t on_set(const std::string&, bool) { return 0; }

  private:
    std::string type_;
    std::vector<Prop> props_;
    std::map<std::string, std::unique_ptr<Buffer>> outs_;

    void collect(const Json& obj, const std::string& prefix, std::vector<std::string>& warnings,
                 std::vector<std::pair<Prop*, const Json*>>& todo) {
        for (const auto& kv : obj.o) {
            const std::string key = prefix + kv.first;
            Prop* p = nullptr;
            for (auto& q : props_)
                if (q.key == key) p = &q;
            if (p) {
                todo.emplace_back(p, &kv.second);
                continue;
            }
            bool group = false;
            for (auto& q : props_)
                group |= q.key.compare(0, key.size() + 1, key + "/") == 0;
            if (group && kv.second.type == Json::Obj) {
                collect(kv.second, key + "/", warnings, todo);
                continue;
            }
            warnings.push_back(type_ + ": property \"" + key + "\" is not known; ignored");
        }
    }
    void check_type(const Prop& p, const Json& v) const {
        const std::string where = type_ + ": property \"" + p.key + "\"";
        switch (p.kind) {
        case Prop::Bool:
            if (v.type != Json::Bool) throw NodeError(where + " must be true or false");
            break;
        case Prop::Int:
            if (v.type != Json::Num || v.n != std::floor(v.n) || std::fabs(v.n) > 9.0e15)
                throw NodeError(where + " must be an integer");
            break;
        case Prop::Float:
            if (v.type != Json::Num) throw NodeError(where + " must be a number");
            break;
        case Prop::Text:
            if (v.type != Json::Str) throw NodeError(where + " must be a string");
            break;
        case Prop::Options:
            if (v.type != Json::Str ||
                std::find(p.options.begin(), p.options.end(), v.s) == p.options.end())
                throw NodeError(where + ": unknown option");
            break;
        }
    }
    static bool same(const Json& a, const Json& c) {
        if (a.type != c.type) return false;
        switch (a.type) {
        case Json::Bool: return a.b == c.b;
        case Json::Num: return a.n == c.n;
        case Json::Str: return a.s == c.s;
        default: return false;
        }
    }
};

const Buffer* input(const std::map<std::string, const Buffer*>& in, const char* name) {
    auto it = in.find(name);
    return it == in.end() ? nullptr : it->second;
}

constexpr const char* kRGBA32F = "R32G32B32A32Sfloat";

// The scene and camera a node renders: its "scene" input when connected, else the graph's.
void scene_of(const std::map<std::string, const Buffer*>& in, uint32_t& scene,
              const gbpt_camera*& camera) {
    const Buffer* sc = input(in, "scene");
    if (sc && sc->is_scene) {
        scene = sc->scene;
        camera = &sc->camera;
    }
    if (!camera) throw NodeError("no camera: connect a scene node or pass a camera");
}

// ---- GBuffer (Raytraced) ---------------------------------------------------------------------
// Outputs "gbuffer" (gbpt_gbuffer_texel per pixel) and "emission" (RGBA32F) at width x height
// (defaults 1920 x 1080, gbuffer_rt.hpp), instance mask bits "0".."7".
class GBufferNode : public Node {
  public:
    GBufferNode() : Node("GBuffer (Raytraced)") {
        add(Prop::Int, "width", jnum(1920), {}, true);
        add(Prop::Int, "height", jnum(1080), {}, true);
        add_mask();
        add(Prop::Options, "emission format", jstr(kRGBA32F), {kRGBA32F}, true);
    }
    std::vector<std::string> inputs() const override { return {"scene"}; }
    std::vector<std::string> outputs() const override { return {"gbuffer", "emission"}; }
    void validate(const std::string& key, const Json& v) override {
        if ((key == "width" || key == "height") && !(v.n >= 1 && v.n <= 65536))
            throw NodeError(type() + ": width and height must be in [1, 65536]");
    }
    void connect(gbpt_ctx*, const std::map<std::string, const Buffer*>&, uint32_t, uint32_t,
                 std::vector<std::string>&) override {
        const uint32_t w = (uint32_t)i("width"), h = (uint32_t)i("height");
        out("gbuffer").allocate(w, h, sizeof(gbpt_gbuffer_texel) / sizeof(float));
        out("emission").allocate(w, h, 4);
    }
    void process(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera, uint64_t,
                 const std::map<std::string, const Buffer*>& in,
                 std::vector<std::string>&) override {
        scene_of(in, scene, camera);
        Buffer& g = out("gbuffer");
        auto* texels = (gbpt_gbuffer_texel*)g.dev;
        check_rc(gbpt_gbuffer(ctx, scene, camera, g.width, g.height, mask(), texels));
        check_rc(gbuffer_emission(ctx, texels, (float*)out("emission").dev, g.texels()));
    }
};

// ---- Render (Path-traced) --------------------------------------------------------------------
// render_pt.cpp:147-186 keys and render_pt.hpp defaults, plus "next event estimation" and
// "russian roulette depth" (off: merian's estimator) and "seed" (RNG lane 3 = seed + the graph
// iteration; 0 is merian's frame counter). The irradiance image has the GBuffer's extent, or the
// graph's extent when no GBuffer is connected.
class RenderPTNode : public Node {
  public:
    RenderPTNode() : Node("Render (Path-traced)") {
        add(Prop::Int, "samples per pixel", jnum(1));
        add(Prop::Int, "max path length", jnum(5));
        add(Prop::Bool, "emission on primary", jbool(true));
        add(Prop::Bool, "shader execution reordering", jbool(false));
        add(Prop::Bool, "demodulate albedo", jbool(false));
        add_mask();
        add(Prop::Options, "irradiance format", jstr(kRGBA32F), {kRGBA32F}, true);
        add(Prop::Bool, "next event estimation", jbool(false));
        add(Prop::Int, "russian roulette depth", jnum(0));
        add(Prop::Int, "seed", jnum(0));
    }
    std::vector<std::string> inputs() const override { return {"scene", "gbuffer"}; }
    std::vector<std::string> outputs() const override { return {"irradiance"}; }
    void validate(const std::string& key, const Json& v) override {
        if (key == "samples per pixel" && !(v.n >= 0 && v.n <= (double)(1u << 24)))
            throw NodeError(type() + ": samples per pixel must be in [0, 2^24]");
        if (key == "max path length" && !(v.n >= 1 && v.n <= 64))
            throw NodeError(type() + ": max path length must be in [1, 64]");
        if (key == "russian roulette depth" && !(v.n >= 0 && v.n <= 64))
            throw NodeError(type() + ": russian roulette depth must be in [0, 64]");
        if (key == "seed" && !(v.n >= 0 && v.n <= 4294967295.0))
            throw NodeError(type() + ": seed must be in [0, 2^32)");
    }
    void connect(gbpt_ctx*, const std::map<std::string, const Buffer*>& in, uint32_t width,
                 uint32_t height, std::vector<std::string>&) override {
        const Buffer* g = input(in, "gbuffer");
        if (g) {
            width = g->width;
            height = g->height;
        }
        out("irradiance").allocate(width, height, 4);
    }
    void process(gbpt_ctx* ctx, uint32_t scene, const gbpt_camera* camera, uint64_t iteration,
                 const std::map<std::string, const Buffer*>& in,
                 std::vector<std::string>&) override {
        scene_of(in, scene, camera);
        Buffer& o = out("irradiance");
        gbpt_render_params p{};
        p.width = o.width;
        p.height = o.height;
        p.spp = (int32_t)i("samples per pixel");
        p.max_path_length = (int32_t)i("max path length");
        p.emission_on_primary = b("emission on primary");
        p.instance_mask = mask();
        p.demodulate_albedo = b("demodulate albedo");
        p.sort_materials = b("shader execution reordering");
        p.frame = (uint32_t)((uint64_t)i("seed") + iteration);
        p.nee = b("next event estimation");
        p.rr_depth = (int32_t)i("russian roulette depth");
        check_rc(gbpt_render_device(ctx, scene, camera, &p, (float*)o.dev, nullptr));
    }
};

// ---- Accumulate --------------------------------------------------------------------------------
// accumulate.cpp:172-250 keys, accumulate.hpp defaults. Static camera: the reprojection settings
// leave the result unchanged (zero motion), so any value is kept; the firefly filter, a finite
// hard clamp and adaptive alpha reduction are not implemented and accept their defaults only.
// The clear at graph iteration 0 and on "clear" follow accumulate.cpp:154-157.
class AccumulateNode : public Node {
  public:
    AccumulateNode() : Node("Accumulate") {
        add(Prop::Float, "alpha", jnum(0.0));
        add(Prop::Float, "max history", jnum(INFINITY));
        add(Prop::Bool, "inf history", jbool(false));
        add(Prop::Bool, "clear", jbool(false));
        add(Prop::Text, "clear event pattern", jstr("/user/clear"), {}, true);
        add(Prop::Bool, "use motion vectors", jbool(true), {}, true);
        add(Prop::Options, "gbuffer check", jstr("always"), {"always", "only if moving", "never"},
            true);
        add(Prop::Float, "normal threshold", jnum(std::acos(0.8) * 180.0 / M_PI));
        add(Prop::Float, "depth threshold", jnum(0.02));
        add(Prop::Options, "filter mode", jstr("nearest"), {"nearest", "stochastic bilinear"},
            true);
        add(Prop::Bool, "extended search", jbool(true), {}, true);
        add(Prop::Bool, "reuse border", jbool(false), {}, true);
        add(Prop::Bool, "firefly filter enable", jbool(false));
        add(Prop::Float, "firefly filter bias", jnum(0.2));
        add(Prop::Float, "IPR factor", jnum(50));
        add(Prop::Float, "firefly percentile lower", jnum(0.25));
        add(Prop::Float, "firefly percentile upper", jnum(0.90));
        add(Prop::Float, "hard clamp", jnum(INFINITY));
        add(Prop::Bool, "inf clamp", jbool(false));
        add(Prop::Float, "adaptivity", jnum(0.0));
        add(Prop::Float, "adaptivity IPR factor", jnum(1.5));
        add(Prop::Float, "adaptivity percentile lower", jnum(0.05));
        add(Prop::Float, "adaptivity percentile upper", jnum(0.95));
        add(Prop::Options, "overwrite format", jstr("Undefined"), {"Undefined", kRGBA32F}, true);
    }
    std::vector<std::string> inputs() const override { return {"src", "gbuffer", "mv"}; }
    std::vector<std::string> outputs() const override { return {"out", "history"}; }
    void validate(const std::string& key, const Json& v) override {
        if (key == "alpha" && !(v.n >= 0 && v.n <= 1))
            throw NodeError(type() + ": alpha must be in [0, 1]");
        if (key == "max history" && !(v.n >= 1))
            throw NodeError(type() + ": max history must be at least 1");
        if (key == "firefly filter enable" && v.b)
            throw NodeError(type() + ": the firefly filter is not implemented in this library");
        if (key == "hard clamp" && std::isfinite(v.n))
            throw NodeError(type() + ": a finite hard clamp is not implemented in this library");
        if (key == "adaptivity" && v.n != 0.0)
            throw NodeError(type() + ": adaptive alpha reduction is not implemented in this "
                                     "build");
    }
    uint32_t on_set(const std::string& key, bool) override {
        // "inf history", "clear" and "inf clamp" are buttons: true acts once
        if (key == "inf history" && b(key)) {
            set("max history", jnum(INFINITY));
            set(key, jbool(false));
        }
        if (key == "clear" && b(key)) {
            clear_ = true;
            set(key, jbool(false));
        }
        if (key == "inf clamp") set(key, jbool(false));
        return 0;
    }
    void connect(gbpt_ctx*, const std::map<std::string, const Buffer*>& in, uint32_t, uint32_t,
                 std::vector<std::string>&) override {
        const Buffer* src = input(in, "src");
        if (!src || src->floats != 4 || src->on_host)
            throw NodeError(type() + ": input \"src\" must be connected to an RGBA32F image");
        Buffer& o = out("out");
        if (o.width != src->width || o.height != src->height) clear_ = true;
        o.allocate(src->width, src->height, 4);
        out("history").allocate(src->width, src->height, 1);
        if (!pending_out_.empty()) {
            if (pending_w_ != src->width || pending_h_ != src->height)
                throw NodeError(type() + ": the checkpoint's extent differs from the input's");
            if (cudaMemcpy(o.dev, pending_out_.data(), pending_out_.size() * sizeof(float),
                           cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(out("history").dev, pending_hist_.data(),
                           pending_hist_.size() * sizeof(float),
                           cudaMemcpyHostToDevice) != cudaSuccess)
                throw NodeError(type() + ": restoring the checkpoint failed");
            pending_out_.clear();
            pending_hist_.clear();
            clear_ = pending_clear_;
        }
    }
    // The accumulated image as two 3-channel PFM files (exact float32): base.rgb.pfm = out.rgb,
    // base.aux.pfm = (out.a, history, 0).
    Json save_state(gbpt_ctx* ctx, const std::string& base) override {
        Json st;
        st.type = Json::Obj;
        st.o.emplace_back("clear", jbool(clear_));
        Buffer* o = output("out");
        if (!o || !o->dev || !ctx) return st;
        std::vector<float> img(o->texels() * 4), hist(o->texels());
        check_rc(gbpt_synchronize(ctx));
        if (cudaMemcpy(img.data(), o->dev, img.size() * sizeof(float), cudaMemcpyDeviceToHost) !=
                cudaSuccess ||
            cudaMemcpy(hist.data(), output("history")->dev, hist.size() * sizeof(float),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            throw NodeError(type() + ": reading the accumulator failed");
        std::vector<float> aux(o->texels() * 3, 0.0f);
        for (uint64_t t = 0; t < o->texels(); ++t) {
            aux[3 * t] = img[4 * t + 3];
            aux[3 * t + 1] = hist[t];
        }
        check_rc(gbpt_image_write_pfm((base + ".rgb.pfm").c_str(), img.data(), o->width,
                                      o->height, 4));
        check_rc(gbpt_image_write_pfm((base + ".aux.pfm").c_str(), aux.data(), o->width,
                                      o->height, 3));
        st.o.emplace_back("width", jnum(o->width));
        st.o.emplace_back("height", jnum(o->height));
        return st;
    }
    void load_state(const Json& st, const std::string& base) override {
        if (st.type != Json::Obj) return;
        const Json* w = st.get("width");
        pending_clear_ = st.get("clear") && st.get("clear")->b;
        clear_ = pending_clear_;
        if (!w) return;
        uint32_t pw = 0, ph = 0;
        check_rc(gbpt_image_read_pfm((base + ".rgb.pfm").c_str(), nullptr, 4, &pw, &ph));
        std::vector<float> rgb((size_t)pw * ph * 4), aux((size_t)pw * ph * 3);
        check_rc(gbpt_image_read_pfm((base + ".rgb.pfm").c_str(), rgb.data(), 4, &pw, &ph));
        uint32_t aw = 0, ah = 0;
        check_rc(gbpt_image_read_pfm((base + ".aux.pfm").c_str(), nullptr, 3, &aw, &ah));
        if (aw != pw || ah != ph) throw NodeError(type() + ": checkpoint images differ in size");
        check_rc(gbpt_image_read_pfm((base + ".aux.pfm").c_str(), aux.data(), 3, &aw, &ah));
        pending_hist_.assign((size_t)pw * ph, 0.0f);
        for (size_t t = 0; t < pending_hist_.size(); ++t) {
            rgb[4 * t + 3] = aux[3 * t];
            pending_hist_[t] = aux[3 * t + 1];
        }
        pending_out_ = std::move(rgb);
        pending_w_ = pw;
        pending_h_ = ph;
    }
    void process(gbpt_ctx* ctx, uint32_t, const gbpt_camera*, uint64_t iteration,
                 const std::map<std::string, const Buffer*>& in,
                 std::vector<std::string>&) override {
        const Buffer* src = input(in, "src");
        Buffer& o = out("out");
        const bool clear = iteration == 0 || clear_;
        check_rc(gbpt_accumulate(ctx, (const float*)src->dev, (float*)o.dev,
                                 (float*)out("history").dev, o.texels(), (float)f("alpha"),
                                 (float)f("max history"), clear));
        clear_ = false;
    }

  private:
    bool clear_ = true;
    bool pending_clear_ = false;
    std::vector<float> pending_out_, pending_hist_;
    uint32_t pending_w_ = 0, pending_h_ = 0;
};

// ---- Image Write -------------------------------------------------------------------------------
// image_write.cpp:60-380 with image_write.hpp's defaults: recording starts when "enable" turns
// true (or at "start at run"), stops on the stop triggers, and with the iteration trigger captures
// when the node's 1-indexed iteration equals "iteration", which is then multiplied by "iteration
// power" and increased by "iteration offset"; "record_next" captures the next iteration. The
// filename is a format string over the node's variables (get_format_args, image_write.hpp:40-63)
// with the format's extension appended; the file is written to a temporary name and renamed.
// PFM only; the frametime trigger, scaling, and the exit triggers accept their defaults only.
class ImageWriteNode : public Node {
  public:
    ImageWriteNode() : Node("Image Write") {
        add(Prop::Options, "format", jstr("PNG"), {"PNG", "JPG", "HDR", "PFM"});
        add(Prop::Text, "filename", jstr("image_{image_index_total:04}"));
        add(Prop::Bool, "record_next", jbool(false));
        add(Prop::Bool, "enable", jbool(false));
        add(Prop::Options, "trigger", jstr("iteration"), {"iteration", "frametime"});
        add(Prop::Int, "iteration", jnum(1));
        add(Prop::Int, "iteration power", jnum(1));
        add(Prop::Int, "iteration offset", jnum(1));
        add(Prop::Bool, "reset iteration at stop", jbool(true));
        add(Prop::Options, "time reference", jstr("system"), {"system", "graph"});
        add(Prop::Float, "framerate", jnum(30));
        add(Prop::Float, "frametime", jnum(1000.0 / 30.0));
        add(Prop::Float, "advanced/scale", jnum(1.0));
        add(Prop::Bool, "advanced/rebuild after capture", jbool(false));
        add(Prop::Bool, "advanced/rebuild on record", jbool(false));
        add(Prop::Bool, "advanced/callback after capture", jbool(false));
        add(Prop::Bool, "advanced/callback on record", jbool(false));
        add(Prop::Int, "advanced/start at run", jnum(-1));
        add(Prop::Int, "advanced/stop at run", jnum(-1));
        add(Prop::Int, "advanced/stop after iteration", jnum(-1));
        add(Prop::Int, "advanced/stop after number captures", jnum(-1));
        add(Prop::Float, "advanced/stop after seconds", jnum(-1));
        add(Prop::Int, "advanced/exit at run", jnum(-1));
        add(Prop::Int, "advanced/exit at iteration", jnum(-1));
        add(Prop::Float, "advanced/exit after seconds", jnum(-1));
    }
    std::vector<std::string> inputs() const override { return {"src"}; }
    std::vector<std::string> outputs() const override { return {}; }
    void validate(const std::string& key, const Json& v) override {
        if (key == "format" && v.s != "PFM")
            throw NodeError(type() + ": format " + v.s + " is not supported (PFM only)");
        if (key == "trigger" && v.s != "iteration")
            throw NodeError(type() + ": the frametime trigger is not supported");
        if (key == "advanced/scale" && v.n != 1.0)
            throw NodeError(type() + ": scaled captures are not supported");
        if ((key == "advanced/stop after seconds" || key == "advanced/exit at run" ||
             key == "advanced/exit at iteration" || key == "advanced/exit after seconds") &&
            v.n != -1.0)
            throw NodeError(type() + ": \"" + key + "\" is not supported");
    }
    uint32_t on_set(const std::string& key, bool changed) override {
        if (key == "record_next") {
            record_next_ |= b(key);
            set(key, jbool(false));
        }
        if (key == "enable") {
            // a value other than the recording state requests a start or stop, carried out
            // before the next capture (pre_process); the value reads as the state until then
            start_stop_ = changed;
            if (changed) set(key, jbool(!b(key)));
        }
        if (key == "iteration") set(key, jnum(std::max<int64_t>(i(key), 0)));
        return 0;
    }
    void connect(gbpt_ctx*, const std::map<std::string, const Buffer*>& in, uint32_t, uint32_t,
                 std::vector<std::string>&) override {
        const Buffer* src = input(in, "src");
        if (!src || src->on_host || (src->floats != 4 && src->floats != 1))
            throw NodeError(type() + ": input \"src\" must be connected to an image");
        if (s("format") != "PFM") // merian's default is PNG
            throw NodeError(type() + ": format " + s("format") +
                            " is not supported (PFM only): set \"format\": \"PFM\"");
    }
    void process(gbpt_ctx* ctx, uint32_t, const gbpt_camera*, uint64_t run_iteration,
                 const std::map<std::string, const Buffer*>& in,
                 std::vector<std::string>& warnings) override {
        pre_process(run_iteration);
        struct Defer {
            int64_t& it;
            ~Defer() { ++it; }
        } defer{iteration_};
        const bool recording = b("enable");
        record_next_ |= recording && i("iteration") == iteration_;
        const Buffer* src = input(in, "src");
        std::string path;
        if (!format_path(src, run_iteration, path)) {
            set("enable", jbool(false));
            record_next_ = false;
            warnings.push_back(type() + ": invalid filename format \"" + s("filename") + "\"");
            return;
        }
        if (!record_next_) return;
        std::vector<float> host(src->texels() * src->floats);
        check_rc(gbpt_synchronize(ctx));
        if (!host.empty() && cudaMemcpy(host.data(), src->dev, host.size() * sizeof(float),
                                        cudaMemcpyDeviceToHost) != cudaSuccess)
            throw NodeError(type() + ": reading the image failed");
        make_parents(path);
        const size_t slash = path.find_last_of('/');
        const std::string tmp = slash == std::string::npos
                                    ? ".interm_" + path
                                    : path.substr(0, slash + 1) + ".interm_" + path.substr(slash + 1);
        check_rc(gbpt_image_write_pfm(tmp.c_str(), host.data(), src->width, src->height,
                                      src->floats));
        if (std::rename(tmp.c_str(), path.c_str()) != 0)
            throw NodeError(type() + ": cannot rename " + tmp + " to " + path);
        record_next_ = false;
        ++captures_since_record_;
        ++captures_total_;
        const int64_t it = i("iteration");
        const int64_t next = recording ? it * i("iteration power") + i("iteration offset") : it;
        set("iteration", jnum((double)next));
    }

    Json save_state(gbpt_ctx*, const std::string&) override {
        Json st;
        st.type = Json::Obj;
        st.o.emplace_back("recording", jbool(b("enable")));
        st.o.emplace_back("record_next", jbool(record_next_));
        st.o.emplace_back("start_stop", jbool(start_stop_));
        st.o.emplace_back("iteration", jnum((double)iteration_));
        st.o.emplace_back("captures_since_record", jnum((double)captures_since_record_));
        st.o.emplace_back("captures_total", jnum((double)captures_total_));
        st.o.emplace_back("iteration_at_start", jnum((double)iteration_at_start_));
        return st;
    }
    void load_state(const Json& st, const std::string&) override {
        if (st.type != Json::Obj) return;
        auto num = [&](const char* k, int64_t def) { return (int64_t)st.num(k, (double)def); };
        const Json* rec = st.get("recording");
        set("enable", jbool(rec && rec->b));
        const Json* rn = st.get("record_next");
        const Json* ss = st.get("start_stop");
        record_next_ = rn && rn->b;
        start_stop_ = ss && ss->b;
        iteration_ = num("iteration", 0);
        captures_since_record_ = num("captures_since_record", 0);
        captures_total_ = num("captures_total", 0);
        iteration_at_start_ = num("iteration_at_start", 1);
    }

  private:
    bool record_next_ = false;
    bool start_stop_ = false;
    int64_t iteration_ = 0;
    int64_t captures_since_record_ = 0;
    int64_t captures_total_ = 0;
    int64_t iteration_at_start_ = 1;
    double record_start_ = 0.0;

    void pre_process(uint64_t run_iteration) {
        bool recording = b("enable");
        if (!recording && (start_stop_ || (int64_t)run_iteration == i("advanced/start at run"))) {
            // record(): start recording
            set("enable", jbool(true));
            recording = true;
            iteration_ = 1;
            captures_since_record_ = 0;
            iteration_at_start_ = i("iteration");
            record_start_ = host_clock();
            start_stop_ = false;
        }
        if (recording &&
            (start_stop_ || i("advanced/stop at run") == (int64_t)run_iteration ||
             (i("advanced/stop after iteration") >= 0 &&
              i("advanced/stop after iteration") < iteration_) ||
             i("advanced/stop after number captures") == captures_since_record_)) {
            set("enable", jbool(false));
            start_stop_ = false;
            captures_since_record_ = 0;
            iteration_ = 1;
            if (b("reset iteration at stop")) set("iteration", jnum((double)iteration_at_start_));
        }
    }

    // fmt-style replacement fields {name} and {name:spec} (spec: [0][width][.precision][type],
    // type d, f, e, g or x), {{ and }} for braces.
    bool format_path(const Buffer* src, uint64_t run_iteration, std::string& path) const {
        const std::string& f = s("filename");
        if (f.empty()) return false;
        const double since = iteration_ > 0 ? host_clock() - record_start_ : 0.0;
        auto lookup = [&](const std::string& name, double& v, bool& integer) {
            integer = true;
            if (name == "record_iteration") v = (double)iteration_;
            else if (name == "image_index_total") v = (double)captures_total_;
            else if (name == "image_index_record") v = (double)captures_since_record_;
            else if (name == "run_iteration") v = (double)run_iteration;
            else if (name == "input_width" || name == "output_width" || name == "width")
                v = src->width;
            else if (name == "input_height" || name == "output_height" || name == "height")
                v = src->height;
            else if (name == "random") v = (double)std::rand();
            else if (name == "graph_time" || name == "graph_time_since_record" ||
                     name == "system_time_since_record" || name == "time") {
                v = since;
                integer = false;
            } else
                return false;
            return true;
        };
        path.clear();
        for (size_t k = 0; k < f.size(); ++k) {
            const char c = f[k];
            if (c == '}') {
                if (k + 1 < f.size() && f[k + 1] == '}') {
                    path += '}';
                    ++k;
                    continue;
                }
                return false;
            }
            if (c != '{') {
                path += c;
                continue;
            }
            if (k + 1 < f.size() && f[k + 1] == '{') {
                path += '{';
                ++k;
                continue;
            }
            const size_t close = f.find('}', k);
            if (close == std::string::npos) return false;
            const std::string field = f.substr(k + 1, close - k - 1);
            k = close;
            const size_t colon = field.find(':');
            const std::string name = field.substr(0, colon);
            std::string spec = colon == std::string::npos ? "" : field.substr(colon + 1);
            double v;
            bool integer;
            if (!lookup(name, v, integer)) return false;
            char type = integer ? 'd' : 'g';
            if (!spec.empty() && std::strchr("dfegx", spec.back())) {
                type = spec.back();
                spec.pop_back();
            }
            for (const char sc : spec)
                if (!(sc == '.' || (sc >= '0' && sc <= '9'))) return false;
            char buf[128];
            const std::string fmt = "%" + spec;
            if (type == 'd' || type == 'x') {
                if (!integer || spec.find('.') != std::string::npos) return false;
                std::snprintf(buf, sizeof(buf), (fmt + "lld").c_str(), (long long)v);
                if (type == 'x')
                    std::snprintf(buf, sizeof(buf), (fmt + "llx").c_str(), (long long)v);
            } else {
                std::snprintf(buf, sizeof(buf), (fmt + type).c_str(), v);
            }
            path += buf;
        }
        path += ".pfm";
        return true;
    }

    static void make_parents(const std::string& path) {
        for (size_t k = 1; k < path.size(); ++k)
            if (path[k] == '/') mkdir(path.substr(0, k).c_str(), 0777);
    }
};

// ---- Error Plot ----------------------------------------------------------------------------------
// error_plot.cpp: the per-channel metric of "input" against "reference" ("Metric": MSE, RMSE =
// sqrt of the MSE, MAE; default RMSE) and its history of "History" values. Outputs (host images,
// this library's form of the node's plot): "error" (1 x 1 RGBA: the latest metric) and "history"
// (n x 1 RGBA, oldest first).
class ErrorPlotNode : public Node {
  public:
    ErrorPlotNode() : Node("Error Plot") {
        add(Prop::Options, "Metric", jstr("RMSE"), {"MSE", "RMSE", "MAE"});
        add(Prop::Int, "History", jnum(256));
        add(Prop::Bool, "Reset history", jbool(false));
        add(Prop::Bool, "Logarithmic x-axis", jbool(false));
        add(Prop::Bool, "Logarithmic y-axis", jbool(false));
        add(Prop::Bool, "Auto scale", jbool(true));
        add(Prop::Float, "Min", jnum(0.0));
        add(Prop::Float, "Max", jnum(1.0));
    }
    std::vector<std::string> inputs() const override { return {"reference", "input"}; }
    std::vector<std::string> outputs() const override { return {"error", "history"}; }
    void validate(const std::string& key, const Json& v) override {
        if (key == "History" && !(v.n >= 1 && v.n <= 1e6))
            throw NodeError(type() + ": History must be in [1, 10^6]");
    }
    uint32_t on_set(const std::string& key, bool) override {
        if (key == "Reset history" && b(key)) {
            history_.clear();
            set(key, jbool(false));
        }
        return 0;
    }
    void connect(gbpt_ctx*, const std::map<std::string, const Buffer*>& in, uint32_t, uint32_t,
                 std::vector<std::string>&) override {
        const Buffer* r = input(in, "reference");
        const Buffer* x = input(in, "input");
        if (!r || !x || r->floats != 4 || x->floats != 4 || r->on_host || x->on_host)
            throw NodeError(type() + ": \"reference\" and \"input\" must be RGBA32F images");
        if (r->width != x->width || r->height != x->height)
            throw NodeError("reference and input image extents mismatch");
        Buffer& e = out("error");
        e.on_host = true;
        e.width = e.height = 1;
        e.host.assign(4, 0.0f);
        out("history").on_host = true;
        publish();
    }
    void process(gbpt_ctx* ctx, uint32_t, const gbpt_camera*, uint64_t,
                 const std::map<std::string, const Buffer*>& in,
                 std::vector<std::string>&) override {
        const Buffer* r = input(in, "reference");
        const Buffer* x = input(in, "input");
        double m[8];
        check_rc(gbpt_error_metrics(ctx, (const float*)r->dev, (const float*)x->dev, r->texels(),
                                    m));
        const std::string& metric = s("Metric");
        Rgba e;
        for (int c = 0; c < 4; ++c) {
            const double v = metric == "MAE" ? m[4 + c] : m[c];
            e.v[c] = metric == "RMSE" ? (float)std::sqrt(std::max(v, 0.0)) : (float)v;
        }
        history_.push_back(e);
        while (history_.size() > (size_t)i("History")) history_.erase(history_.begin());
        publish();
    }

    Json save_state(gbpt_ctx*, const std::string&) override {
        Json st;
        st.type = Json::Arr;
        for (const auto& h : history_)
            for (int c = 0; c < 4; ++c) st.a.push_back(jnum(h.v[c]));
        return st;
    }
    void load_state(const Json& st, const std::string&) override {
        history_.clear();
        for (size_t k = 0; k + 3 < st.size(); k += 4) {
            Rgba r;
            for (int c = 0; c < 4; ++c) r.v[c] = (float)st.a[k + c].n;
            history_.push_back(r);
        }
    }

  private:
    struct Rgba {
        float v[4];
    };
    std::vector<Rgba> history_;

    void publish() {
        Buffer& e = out("error");
        Buffer& h = out("history");
        h.width = (uint32_t)history_.size();
        h.height = history_.empty() ? 0 : 1;
        h.host.clear();
        for (const auto& x : history_) h.host.insert(h.host.end(), x.v, x.v + 4);
        if (!history_.empty()) e.host.assign(history_.back().v, history_.back().v + 4);
    }
};

// ---- GLTF Scene / PBRT Scene ------------------------------------------------------------------------
// nodes/gltf_scene/gltf_scene_node.cpp:38-40,85-100 and nodes/pbrt_scene/pbrt_scene_node.cpp:
// "file" is loaded (gbpt_load_gltf / gbpt_load_pbrt) and made resident on the context when the
// graph connects; the output "scene" carries the scene and the file's camera to the GBuffer and
// renderer nodes. The loaders' warnings join the graph's.
class SceneFileNode : public Node {
  public:
    explicit SceneFileNode(bool gltf) : Node(gltf ? "GLTF Scene" : "PBRT Scene"), gltf_(gltf) {
        add(Prop::Text, "file", jstr(""), {}, true);
    }
    ~SceneFileNode() override { unload(); }
    std::vector<std::string> inputs() const override { return {}; }
    std::vector<std::string> outputs() const override { return {"scene"}; }
    void connect(gbpt_ctx* ctx, const std::map<std::string, const Buffer*>&, uint32_t, uint32_t,
                 std::vector<std::string>& warnings) override {
        Buffer& o = out("scene");
        o.is_scene = true;
        if (o.scene && loaded_file_ == s("file") && ctx_ == ctx) return;
        unload();
        if (s("file").empty()) throw NodeError(type() + ": no \"file\" given");
        gbpt_loaded_scene* ls = nullptr;
        check_rc(gltf_ ? gbpt_load_gltf(s("file").c_str(), &ls)
                       : gbpt_load_pbrt(s("file").c_str(), &ls));
        gbpt_loaded_info info{};
        int rc = gbpt_loaded_scene_info(ls, &info);
        uint32_t id = 0;
        if (rc == GBPT_OK) rc = gbpt_scene_create(ctx, &info.desc, &id);
        for (uint32_t k = 0; rc == GBPT_OK && k < info.warning_count; ++k)
            warnings.push_back(type() + ": " + gbpt_loaded_scene_warning(ls, k));
        gbpt_loaded_scene_free(ls);
        check_rc(rc);
        ctx_ = ctx;
        o.scene = id;
        o.camera = info.camera;
        loaded_file_ = s("file");
    }
    void process(gbpt_ctx*, uint32_t, const gbpt_camera*, uint64_t,
                 const std::map<std::string, const Buffer*>&, std::vector<std::string>&) override {}

  private:
    bool gltf_;
    gbpt_ctx* ctx_ = nullptr;
    std::string loaded_file_;
    void unload() {
        Buffer* o = output("scene");
        if (o && o->scene && ctx_) gbpt_scene_destroy(ctx_, o->scene);
        if (o) o->scene = 0;
    }
};

// ---- registry ----------------------------------------------------------------------------------
using Factory = std::function<std::unique_ptr<Node>()>;

const std::map<std::string, Factory>& registry() {
    static const std::map<std::string, Factory> r = {
        {"Render (Path-traced)", [] { return std::unique_ptr<Node>(new RenderPTNode()); }},
        {"GBuffer (Raytraced)", [] { return std::unique_ptr<Node>(new GBufferNode()); }},
        {"Accumulate", [] { return std::unique_ptr<Node>(new AccumulateNode()); }},
        {"Image Write", [] { return std::unique_ptr<Node>(new ImageWriteNode()); }},
        {"Error Plot", [] { return std::unique_ptr<Node>(new ErrorPlotNode()); }},
        {"GLTF Scene", [] { return std::unique_ptr<Node>(new SceneFileNode(true)); }},
        {"PBRT Scene", [] { return std::unique_ptr<Node>(new SceneFileNode(false)); }},
    };
    return r;
}

struct Edge {
    std::string src, output, dst, input;
};

} // namespace
} // namespace gbpt

using namespace gbpt;

struct gbpt_graph {
    gbpt_ctx* ctx = nullptr;
    std::map<std::string, std::unique_ptr<Node>> nodes;
    std::vector<std::string> order; // dependency order, ties by name
    std::vector<Edge> edges;
    std::vector<std::string> warnings;
    // the graph JSON's "cli" options (main.cpp:31-51): option name -> JSON pointer, and the node
    // and property key ("group/key") the pointer addresses
    struct Option {
        std::string name, pointer, node, key;
    };
    std::vector<Option> options;
    bool connected = false;
    uint32_t width = 0, height = 0; // the extent of the last connect
    uint64_t iteration = 0;         // graph iterations run so far

    std::map<std::string, const Buffer*> inputs_of(const std::string& name) {
        std::map<std::string, const Buffer*> in;
        for (const auto& e : edges)
            if (e.dst == name) in[e.input] = nodes[e.src]->output(e.output);
        return in;
    }
};

namespace {

int fail(const std::string& msg, int rc = GBPT_ERR_INVALID) {
    set_error(msg);
    return rc;
}

template <class F> int guarded(const char* fn, F&& body) {
    try {
        return body();
    } catch (const NodeError& e) {
        return fail(std::string(fn) + ": " + e.what());
    } catch (const std::bad_alloc&) {
        return fail(std::string(fn) + ": out of memory", GBPT_ERR_NO_MEMORY);
    } catch (const std::exception& e) {
        return fail(std::string(fn) + ": " + e.what());
    }
}

void topological(gbpt_graph& g) {
    std::map<std::string, std::set<std::string>> deps;
    for (const auto& n : g.nodes) deps[n.first];
    for (const auto& e : g.edges) deps[e.dst].insert(e.src);
    std::set<std::string> done;
    g.order.clear();
    while (g.order.size() < g.nodes.size()) {
        std::vector<std::string> ready;
        for (const auto& d : deps)
            if (!done.count(d.first) &&
                std::includes(done.begin(), done.end(), d.second.begin(), d.second.end()))
                ready.push_back(d.first);
        if (ready.empty()) throw NodeError("the graph has a cycle");
        for (const auto& r : ready) {
            g.order.push_back(r);
            done.insert(r);
        }
    }
}

Node* find_node(gbpt_graph* g, const char* name) {
    if (!g || !name) return nullptr;
    auto it = g->nodes.find(name);
    return it == g->nodes.end() ? nullptr : it->second.get();
}

} // namespace

extern "C" {

GBPT_API int gbpt_graph_create(gbpt_ctx* ctx, const char* graph_json, gbpt_graph** out_graph) {
    if (!graph_json || !out_graph) return fail("gbpt_graph_create: null argument");
    *out_graph = nullptr;
    return guarded("gbpt_graph_create", [&]() -> int {
        Json root;
        std::string err;
        if (!parse_json(graph_json, root, err)) throw NodeError(err);
        const Json* nodes = root.get("nodes");
        if (root.type != Json::Obj || !nodes || nodes->type != Json::Obj)
            throw NodeError("the graph JSON has no \"nodes\" object");
        std::unique_ptr<gbpt_graph> g(new gbpt_graph());
        g->ctx = ctx;
        std::vector<std::pair<std::string, std::string>> raw_edges;
        for (const auto& kv : nodes->o) {
            const Json& spec = kv.second;
            if (spec.type != Json::Obj) throw NodeError("node \"" + kv.first + "\": not an object");
            const Json* en = spec.get("enabled");
            if (en && en->type == Json::Bool && !en->b) continue;
            const std::string type = spec.str("type", "");
            auto f = registry().find(type);
            if (f == registry().end())
                throw NodeError("node \"" + kv.first + "\": type \"" + type +
                                "\" is not available in this library");
            if (g->nodes.count(kv.first)) throw NodeError("node \"" + kv.first + "\" twice");
            std::unique_ptr<Node> node = f->second();
            if (const Json* props = spec.get("properties"))
                node->set_properties(*props, g->warnings);
            if (const Json* outs = spec.get("outputs")) {
                if (outs->type != Json::Arr)
                    throw NodeError("node \"" + kv.first + "\": \"outputs\" must be a list");
                for (const auto& e : outs->a) {
                    if (e.type != Json::Str) throw NodeError("node \"" + kv.first + "\": bad edge");
                    raw_edges.emplace_back(kv.first, e.s);
                }
            }
            g->nodes[kv.first] = std::move(node);
        }
        for (const auto& re : raw_edges) {
            const size_t arrow = re.second.find("->");
            const size_t dot = re.second.rfind('.');
            if (arrow == std::string::npos || dot == std::string::npos || dot < arrow)
                throw NodeError("edge \"" + re.second + "\" of node \"" + re.first +
                                "\": expected \"output->node.input\"");
            Edge e{re.first, re.second.substr(0, arrow),
                   re.second.substr(arrow + 2, dot - arrow - 2), re.second.substr(dot + 1)};
            if (!g->nodes.count(e.dst)) {
                g->warnings.push_back("edge \"" + re.second + "\" of node \"" + re.first +
                                      "\" leads to a node that is absent or disabled; ignored");
                continue;
            }
            const auto outs = g->nodes[e.src]->outputs();
            const auto ins = g->nodes[e.dst]->inputs();
            if (std::find(outs.begin(), outs.end(), e.output) == outs.end())
                throw NodeError("node \"" + e.src + "\" has no output \"" + e.output + "\"");
            if (std::find(ins.begin(), ins.end(), e.input) == ins.end())
                throw NodeError("node \"" + e.dst + "\" has no input \"" + e.input + "\"");
            for (const auto& o : g->edges)
                if (o.dst == e.dst && o.input == e.input)
                    throw NodeError("input \"" + e.dst + "." + e.input + "\" connected twice");
            g->edges.push_back(e);
        }
        if (const Json* cli = root.get("cli")) {
            for (const auto& kv : cli->o) {
                const std::string ptr = kv.second.str("pointer", "");
                // RFC 6901 tokens: "~1" is "/", "~0" is "~"
                std::vector<std::string> tok;
                for (size_t at = 0; at < ptr.size() && ptr[at] == '/';) {
                    const size_t next = ptr.find('/', at + 1);
                    std::string t = ptr.substr(at + 1, next == std::string::npos ? std::string::npos
                                                                                  : next - at - 1);
                    for (size_t q; (q = t.find("~1")) != std::string::npos;) t.replace(q, 2, "/");
                    for (size_t q; (q = t.find("~0")) != std::string::npos;) t.replace(q, 2, "~");
                    tok.push_back(t);
                    if (next == std::string::npos) break;
                    at = next;
                }
                if (tok.size() < 4 || tok[0] != "nodes" || tok[2] != "properties" ||
                    !g->nodes.count(tok[1])) {
                    g->warnings.push_back("cli option \"" + kv.first + "\": pointer \"" + ptr +
                                          "\" does not name a property of an enabled node");
                    continue;
                }
                std::string key = tok[3];
                for (size_t k = 4; k < tok.size(); ++k) key += "/" + tok[k];
                if (!g->nodes[tok[1]]->prop(key)) {
                    g->warnings.push_back("cli option \"" + kv.first + "\": node \"" + tok[1] +
                                          "\" has no property \"" + key + "\"");
                    continue;
                }
                g->options.push_back({kv.first, ptr, tok[1], key});
            }
        }
        topological(*g);
        *out_graph = g.release();
        return GBPT_OK;
    });
}

GBPT_API int gbpt_graph_destroy(gbpt_graph* graph) {
    if (!graph) return GBPT_OK;
    if (graph->ctx) {
        gbpt_synchronize(graph->ctx);
        cudaSetDevice(graph->ctx->device);
    }
    delete graph;
    return GBPT_OK;
}

GBPT_API int gbpt_graph_node_count(const gbpt_graph* graph, uint32_t* count) {
    if (!graph || !count) return fail("gbpt_graph_node_count: null argument");
    *count = (uint32_t)graph->order.size();
    return GBPT_OK;
}

GBPT_API int gbpt_graph_node(const gbpt_graph* graph, uint32_t index, const char** name,
                             const char** type) {
    if (!graph || index >= graph->order.size())
        return fail("gbpt_graph_node: null graph or index out of range");
    const std::string& n = graph->order[index];
    if (name) *name = n.c_str();
    if (type) *type = graph->nodes.at(n)->type().c_str();
    return GBPT_OK;
}

GBPT_API uint32_t gbpt_graph_warning_count(const gbpt_graph* graph) {
    return graph ? (uint32_t)graph->warnings.size() : 0u;
}

GBPT_API const char* gbpt_graph_warning(const gbpt_graph* graph, uint32_t index) {
    return graph && index < graph->warnings.size() ? graph->warnings[index].c_str() : nullptr;
}

GBPT_API int gbpt_graph_set_property(gbpt_graph* graph, const char* node, const char* key,
                                     const char* json_value, uint32_t* out_flags) {
    Node* n = find_node(graph, node);
    if (!n || !key || !json_value)
        return fail("gbpt_graph_set_property: null argument or unknown node");
    return guarded("gbpt_graph_set_property", [&]() -> int {
        Json v;
        std::string err;
        if (!parse_json(json_value, v, err)) throw NodeError(err);
        // "group/key" addresses a property inside a group such as "advanced"
        Json obj;
        obj.type = Json::Obj;
        Json* at = &obj;
        std::string k = key;
        for (size_t slash; (slash = k.find('/')) != std::string::npos; k = k.substr(slash + 1)) {
            at->o.emplace_back(k.substr(0, slash), Json());
            at = &at->o.back().second;
            at->type = Json::Obj;
        }
        at->o.emplace_back(k, v);
        std::vector<std::string> unknown;
        const uint32_t flags = n->set_properties(obj, unknown);
        if (!unknown.empty()) throw NodeError(unknown.front());
        if (flags & kNeedsReconnect) graph->connected = false;
        if (out_flags) *out_flags = flags;
        return GBPT_OK;
    });
}

GBPT_API int gbpt_graph_option(const gbpt_graph* graph, uint32_t index, const char** name,
                               const char** pointer) {
    if (!graph) return fail("gbpt_graph_option: null graph");
    if (index >= graph->options.size()) return fail("gbpt_graph_option: no such option",
                                                    GBPT_ERR_NOT_FOUND);
    if (name) *name = graph->options[index].name.c_str();
    if (pointer) *pointer = graph->options[index].pointer.c_str();
    return GBPT_OK;
}

GBPT_API int gbpt_graph_set_option(gbpt_graph* graph, const char* option, const char* json_value,
                                   uint32_t* out_flags) {
    if (!graph || !option) return fail("gbpt_graph_set_option: null argument");
    for (const auto& o : graph->options)
        if (o.name == option)
            return gbpt_graph_set_property(graph, o.node.c_str(), o.key.c_str(), json_value,
                                           out_flags);
    return fail(std::string("gbpt_graph_set_option: no option \"") + option + "\"",
                GBPT_ERR_NOT_FOUND);
}

GBPT_API int gbpt_graph_get_property(const gbpt_graph* graph, const char* node, const char* key,
                                     char* json_out, uint64_t capacity, uint64_t* length) {
    Node* n = find_node(const_cast<gbpt_graph*>(graph), node);
    if (!n) return fail("gbpt_graph_get_property: null graph or unknown node");
    std::string text;
    if (key) {
        const Prop* p = n->prop(key);
        if (!p) return fail(std::string("gbpt_graph_get_property: unknown property ") + key);
        dump_json(p->value, text);
    } else {
        dump_json(n->all_properties(), text);
    }
    if (length) *length = text.size();
    if (json_out && capacity) {
        const size_t c = std::min<size_t>(text.size(), capacity - 1);
        std::memcpy(json_out, text.data(), c);
        json_out[c] = '\0';
        if (c < text.size()) return fail("gbpt_graph_get_property: buffer too small");
    }
    return GBPT_OK;
}

GBPT_API int gbpt_graph_run(gbpt_graph* graph, uint32_t scene, const gbpt_camera* camera,
                            uint32_t width, uint32_t height, uint32_t iterations) {
    if (!graph) return fail("gbpt_graph_run: null graph");
    if (!graph->ctx) return fail("gbpt_graph_run: the graph was created without a context");
    if (width == 0 || height == 0 || width > 65536 || height > 65536)
        return fail("gbpt_graph_run: extent out of range");
    int rc = check_ctx(graph->ctx);
    if (rc) return rc;
    return guarded("gbpt_graph_run", [&]() -> int {
        if (!graph->connected || width != graph->width || height != graph->height) {
            for (const auto& name : graph->order)
                graph->nodes[name]->connect(graph->ctx, graph->inputs_of(name), width, height,
                                            graph->warnings);
            graph->connected = true;
            graph->width = width;
            graph->height = height;
        }
        for (uint32_t it = 0; it < iterations; ++it, ++graph->iteration)
            for (const auto& name : graph->order)
                graph->nodes[name]->process(graph->ctx, scene, camera, graph->iteration,
                                            graph->inputs_of(name), graph->warnings);
        return GBPT_OK;
    });
}

GBPT_API int gbpt_graph_to_json(const gbpt_graph* graph, char* json_out, uint64_t capacity,
                                uint64_t* length) {
    if (!graph) return fail("gbpt_graph_to_json: null graph");
    // merian's layout (graph_load_store.cpp): "cli", then "nodes" by name with "enabled",
    // "outputs" ("output->node.input"), "properties" and "type"
    Json root;
    root.type = Json::Obj;
    if (!graph->options.empty()) {
        Json cli;
        cli.type = Json::Obj;
        for (const auto& o : graph->options) {
            Json e;
            e.type = Json::Obj;
            e.o.emplace_back("pointer", jstr(o.pointer));
            cli.o.emplace_back(o.name, std::move(e));
        }
        root.o.emplace_back("cli", std::move(cli));
    }
    Json nodes;
    nodes.type = Json::Obj;
    for (const auto& kv : graph->nodes) {
        Json e;
        e.type = Json::Obj;
        e.o.emplace_back("enabled", jbool(true));
        Json outs;
        outs.type = Json::Arr;
        for (const auto& ed : graph->edges)
            if (ed.src == kv.first)
                outs.a.push_back(jstr(ed.output + "->" + ed.dst + "." + ed.input));
        e.o.emplace_back("outputs", std::move(outs));
        e.o.emplace_back("properties", kv.second->all_properties());
        e.o.emplace_back("type", jstr(kv.second->type()));
        nodes.o.emplace_back(kv.first, std::move(e));
    }
    root.o.emplace_back("nodes", std::move(nodes));
    std::string text;
    dump_json(root, text);
    if (length) *length = text.size();
    if (json_out && capacity) {
        const size_t c = std::min<size_t>(text.size(), capacity - 1);
        std::memcpy(json_out, text.data(), c);
        json_out[c] = '\0';
        if (c < text.size()) return fail("gbpt_graph_to_json: buffer too small");
    }
    return GBPT_OK;
}

GBPT_API int gbpt_graph_save(gbpt_graph* graph, const char* directory) {
    if (!graph || !directory) return fail("gbpt_graph_save: null argument");
    if (graph->ctx) {
        int rc = check_ctx(graph->ctx);
        if (rc) return rc;
    }
    return guarded("gbpt_graph_save", [&]() -> int {
        const std::string dir = directory;
        mkdir(dir.c_str(), 0777);
        Json root;
        root.type = Json::Obj;
        root.o.emplace_back("iteration", jnum((double)graph->iteration));
        Json nodes;
        nodes.type = Json::Obj;
        for (const auto& name : graph->order) {
            Node& n = *graph->nodes[name];
            Json e;
            e.type = Json::Obj;
            e.o.emplace_back("type", jstr(n.type()));
            e.o.emplace_back("properties", n.all_properties());
            e.o.emplace_back("state", n.save_state(graph->ctx, dir + "/" + name));
            nodes.o.emplace_back(name, std::move(e));
        }
        root.o.emplace_back("nodes", std::move(nodes));
        std::string text;
        dump_json(root, text);
        const std::string path = dir + "/graph_state.json";
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) throw NodeError("cannot write " + path);
        const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
        if (std::fclose(f) != 0 || !ok) throw NodeError("cannot write " + path);
        return GBPT_OK;
    });
}

GBPT_API int gbpt_graph_load(gbpt_graph* graph, const char* directory) {
    if (!graph || !directory) return fail("gbpt_graph_load: null argument");
    return guarded("gbpt_graph_load", [&]() -> int {
        const std::string dir = directory;
        const std::string path = dir + "/graph_state.json";
        FILE* f = std::fopen(path.c_str(), "rb");
        if (!f) throw NodeError("cannot read " + path);
        std::string text;
        char buf[65536];
        size_t n;
        while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
        std::fclose(f);
        Json root;
        std::string err;
        if (!parse_json(text, root, err)) throw NodeError(path + ": " + err);
        const Json* nodes = root.get("nodes");
        if (!nodes || nodes->type != Json::Obj) throw NodeError(path + ": no \"nodes\"");
        for (const auto& kv : nodes->o) {
            Node* node = find_node(graph, kv.first.c_str());
            if (!node || node->type() != kv.second.str("type", ""))
                throw NodeError(path + ": node \"" + kv.first + "\" is not in this graph");
        }
        for (const auto& kv : nodes->o) {
            Node* node = find_node(graph, kv.first.c_str());
            std::vector<std::string> unknown;
            if (const Json* props = kv.second.get("properties"))
                node->set_properties(*props, unknown);
            const Json* st = kv.second.get("state");
            node->load_state(st ? *st : Json(), dir + "/" + kv.first);
        }
        graph->iteration = (uint64_t)root.num("iteration", 0.0);
        graph->connected = false;
        return GBPT_OK;
    });
}

GBPT_API int gbpt_graph_output(gbpt_graph* graph, const char* connector, float* out_host,
                               uint64_t capacity_floats, uint32_t* width, uint32_t* height,
                               uint32_t* floats_per_texel) {
    if (!graph || !connector) return fail("gbpt_graph_output: null argument");
    const std::string c = connector;
    const size_t dot = c.rfind('.');
    Node* n = dot == std::string::npos ? nullptr : find_node(graph, c.substr(0, dot).c_str());
    Buffer* b = n ? n->output(c.substr(dot + 1)) : nullptr;
    if (!b) return fail("gbpt_graph_output: no output \"" + c + "\" (run the graph first)");
    if (width) *width = b->width;
    if (height) *height = b->height;
    if (floats_per_texel) *floats_per_texel = b->floats;
    if (!out_host) return GBPT_OK;
    const uint64_t count = b->texels() * b->floats;
    if (capacity_floats < count) return fail("gbpt_graph_output: buffer too small");
    if (b->on_host) {
        std::copy(b->host.begin(), b->host.begin() + (ptrdiff_t)count, out_host);
        return GBPT_OK;
    }
    int rc = gbpt_synchronize(graph->ctx);
    if (rc) return rc;
    GBPT_CUDA_CHECK(cudaMemcpy(out_host, b->dev, count * sizeof(float), cudaMemcpyDeviceToHost));
    return GBPT_OK;
}

} // extern "C"

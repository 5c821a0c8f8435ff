// A small JSON reader and writer for the host code: glTF files and merian graph JSONs
// (nodes, their properties and edges). Numbers are doubles; objects keep their key order.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace gbpt {

struct Json {
    enum Type { Null, Bool, Num, Str, Arr, Obj } type = Null;
    bool b = false;
    double n = 0.0;
    std::string s;
    std::vector<Json> a;
    std::vector<std::pair<std::string, Json>> o;

    const Json* get(const char* key) const {
        if (type != Obj) return nullptr;
        for (const auto& kv : o)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    double num(const char* key, double def) const {
        const Json* v = get(key);
        return v && v->type == Num ? v->n : def;
    }
    int idx(const char* key) const { // a glTF index, -1 when absent
        const Json* v = get(key);
        return v && v->type == Num ? (int)v->n : -1;
    }
    std::string str(const char* key, const std::string& def) const {
        const Json* v = get(key);
        return v && v->type == Str ? v->s : def;
    }
    size_t size() const { return type == Arr ? a.size() : 0; }
};

class JsonParser {
  public:
    JsonParser(const char* b, const char* e) : p(b), end(e) {}
    bool parse(Json& out, std::string& err) {
        if (!value(out, 0)) {
            err = "JSON syntax error at byte " + std::to_string(offset());
            return false;
        }
        ws();
        return true;
    }
    bool at_end() const { return p == end; }

  private:
    const char* p;
    const char* end;
    const char* begin_ = p;
    size_t offset() const { return (size_t)(p - begin_); }
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool lit(const char* w) {
        const size_t n = std::strlen(w);
        if ((size_t)(end - p) < n || std::strncmp(p, w, n) != 0) return false;
        p += n;
        return true;
    }
    static void utf8(uint32_t c, std::string& s) {
        if (c < 0x80) {
            s += (char)c;
        } else if (c < 0x800) {
            s += (char)(0xC0 | (c >> 6));
            s += (char)(0x80 | (c & 0x3F));
        } else if (c < 0x10000) {
            s += (char)(0xE0 | (c >> 12));
            s += (char)(0x80 | ((c >> 6) & 0x3F));
            s += (char)(0x80 | (c & 0x3F));
        } else {
            s += (char)(0xF0 | (c >> 18));
            s += (char)(0x80 | ((c >> 12) & 0x3F));
            s += (char)(0x80 | ((c >> 6) & 0x3F));
            s += (char)(0x80 | (c & 0x3F));
        }
    }
    bool hex4(uint32_t& v) {
        if (end - p < 4) return false;
        v = 0;
        for (int i = 0; i < 4; ++i) {
            const char c = *p++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else return false;
        }
        return true;
    }
    bool string(std::string& s) {
        if (p >= end || *p != '"') return false;
        ++p;
        while (p < end && *p != '"') {
            if (*p == '\\') {
                if (++p >= end) return false;
                switch (*p++) {
                case '"': s += '"'; break;
                case '\\': s += '\\'; break;
                case '/': s += '/'; break;
                case 'b': s += '\b'; break;
                case 'f': s += '\f'; break;
                case 'n': s += '\n'; break;
                case 'r': s += '\r'; break;
                case 't': s += '\t'; break;
                case 'u': {
                    uint32_t c;
                    if (!hex4(c)) return false;
                    if (c >= 0xD800 && c < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                        p += 2;
                        uint32_t lo;
                        if (!hex4(lo)) return false;
                        c = 0x10000 + ((c - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(c, s);
                    break;
                }
                default: return false;
                }
            } else {
                s += *p++;
            }
        }
        if (p >= end) return false;
        ++p;
        return true;
    }
    bool value(Json& v, int depth) {
        if (depth > 256) return false;
        ws();
        if (p >= end) return false;
        const char c = *p;
        if (c == '{') {
            ++p;
            v.type = Json::Obj;
            ws();
            if (p < end && *p == '}') {
                ++p;
                return true;
            }
            while (true) {
                ws();
                std::string k;
                if (!string(k)) return false;
                ws();
                if (p >= end || *p != ':') return false;
                ++p;
                v.o.emplace_back(std::move(k), Json());
                if (!value(v.o.back().second, depth + 1)) return false;
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == '}') {
                    ++p;
                    return true;
                }
                return false;
            }
        }
        if (c == '[') {
            ++p;
            v.type = Json::Arr;
            ws();
            if (p < end && *p == ']') {
                ++p;
                return true;
            }
            while (true) {
                v.a.emplace_back();
                if (!value(v.a.back(), depth + 1)) return false;
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == ']') {
                    ++p;
                    return true;
                }
                return false;
            }
        }
        if (c == '"') {
            v.type = Json::Str;
            return string(v.s);
        }
        if (lit("true")) {
            v.type = Json::Bool;
            v.b = true;
            return true;
        }
        if (lit("false")) {
            v.type = Json::Bool;
            return true;
        }
        if (lit("null")) return true;
        char* e = nullptr;
        v.n = std::strtod(p, &e);
        if (e == p) return false;
        p = e;
        v.type = Json::Num;
        return true;
    }
};

// Parses the whole text (only white space may follow the value).
inline bool parse_json(const std::string& text, Json& out, std::string& err) {
    JsonParser jp(text.data(), text.data() + text.size());
    if (!jp.parse(out, err)) return false;
    if (!jp.at_end()) {
        err = "JSON: unexpected text after the value";
        return false;
    }
    return true;
}

// Compact JSON text of a value (numbers in the shortest form that reads back exactly).
inline void dump_json(const Json& v, std::string& out) {
    switch (v.type) {
    case Json::Null: out += "null"; break;
    case Json::Bool: out += v.b ? "true" : "false"; break;
    case Json::Num: {
        char buf[40];
        if (!std::isfinite(v.n)) {
            out += "null";
            break;
        }
        for (int prec = 1; prec <= 17; ++prec) {
            std::snprintf(buf, sizeof(buf), "%.*g", prec, v.n);
            if (std::strtod(buf, nullptr) == v.n) break;
        }
        out += buf;
        break;
    }
    case Json::Str: {
        out += '"';
        for (const char c : v.s) {
            if (c == '"' || c == '\\') {
                out += '\\';
                out += c;
            } else if ((unsigned char)c < 0x20) {
                char buf[8];
                std::snprintf(buf, sizeof(buf), "\\u%04x", (unsigned)(unsigned char)c);
                out += buf;
            } else {
                out += c;
            }
        }
        out += '"';
        break;
    }
    case Json::Arr:
        out += '[';
        for (size_t i = 0; i < v.a.size(); ++i) {
            if (i) out += ',';
            dump_json(v.a[i], out);
        }
        out += ']';
        break;
    case Json::Obj:
        out += '{';
        for (size_t i = 0; i < v.o.size(); ++i) {
            if (i) out += ',';
            Json k;
            k.type = Json::Str;
            k.s = v.o[i].first;
            dump_json(k, out);
            out += ':';
            dump_json(v.o[i].second, out);
        }
        out += '}';
        break;
    }
}

} // namespace gbpt

// PNG decoding for the scene loaders' image textures: zlib/DEFLATE (RFC 1950/1951) inflation, the
// five PNG scanline filters and the colour types to RGBA8 (PNG specification, ISO/IEC 15948).
// Bit depths 8 and 16 for grey, RGB, grey+alpha and RGBA (16-bit samples keep their high byte),
// palettes of depth 1, 2, 4 and 8 with an optional tRNS alpha table, no interlacing. Host only.
#include "gbpt.h"
#include "host_common.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace gbpt {
namespace {

// ---- inflate -----------------------------------------------------------------------------------
struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0; // pos in bits
    bool bad = false;
    uint32_t bits(int k) {
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) {
            const size_t byte = pos >> 3;
            if (byte >= n) {
                bad = true;
                return 0;
            }
            v |= (uint32_t)((p[byte] >> (pos & 7)) & 1u) << i;
            ++pos;
        }
        return v;
    }
    void align() { pos = (pos + 7) & ~(size_t)7; }
};

// Canonical Huffman code from code lengths: counts per length and symbols in code order.
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t* len, int n) {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; ++i) count[len[i]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left <<= 1;
            left -= count[l];
            if (left < 0) return false; // over-subscribed
        }
        uint16_t offs[16] = {};
        for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + count[l];
        symbol.assign(n, 0);
        for (int i = 0; i < n; ++i)
            if (len[i]) symbol[offs[len[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (int)br.bits(1);
            if (br.bad) return -1;
            const int c = count[l];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                               2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,
                                33,  49,  65,  97,  129, 193,  257,  385,  513,  769,
                                1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
    while (true) {
        const int sym = lit.decode(br);
        if (sym < 0) return false;
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            const int li = sym - 257;
            if (li >= 29) return false;
            const uint32_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int ds = dist.decode(br);
            if (ds < 0 || ds >= 30) return false;
            const uint32_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (br.bad || d > out.size()) return false;
            const size_t from = out.size() - d;
            for (uint32_t k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

bool inflate_zlib(const uint8_t* p, size_t n, std::vector<uint8_t>& out, std::string& err) {
    if (n < 2 || (p[0] & 0x0F) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20)) {
        err = "bad zlib header";
        return false;
    }
    BitReader br{p + 2, n - 2};
    bool last = false;
    while (!last) {
        last = br.bits(1) != 0;
        const uint32_t type = br.bits(2);
        if (br.bad) break;
        if (type == 0) {
            br.align();
            const size_t byte = br.pos >> 3;
            if (byte + 4 > br.n) break;
            const uint32_t len = br.p[byte] | (br.p[byte + 1] << 8);
            const uint32_t nlen = br.p[byte + 2] | (br.p[byte + 3] << 8);
            if ((len ^ 0xFFFFu) != nlen || byte + 4 + len > br.n) {
                err = "bad stored block";
                return false;
            }
            out.insert(out.end(), br.p + byte + 4, br.p + byte + 4 + len);
            br.pos = (byte + 4 + len) * 8;
        } else if (type == 1) {
            uint8_t len[288 + 32];
            for (int i = 0; i < 144; ++i) len[i] = 8;
            for (int i = 144; i < 256; ++i) len[i] = 9;
            for (int i = 256; i < 280; ++i) len[i] = 7;
            for (int i = 280; i < 288; ++i) len[i] = 8;
            for (int i = 0; i < 30; ++i) len[288 + i] = 5;
            Huffman lit, dist;
            lit.build(len, 288);
            dist.build(len + 288, 30);
            if (!inflate_block(br, lit, dist, out)) {
                err = "corrupt fixed-Huffman block";
                return false;
            }
        } else if (type == 2) {
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1,
                      hclen = (int)br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8,  7, 9,  6, 10, 5,
                                              11, 4,  12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) {
                err = "bad code-length code";
                return false;
            }
            uint8_t len[320] = {};
            int i = 0;
            while (i < hlit + hdist) {
                const int sym = clh.decode(br);
                if (sym < 0) {
                    err = "bad code lengths";
                    return false;
                }
                if (sym < 16) {
                    len[i++] = (uint8_t)sym;
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (i == 0) {
                            err = "repeat without a length";
                            return false;
                        }
                        val = len[i - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (i + rep > hlit + hdist) {
                        err = "code lengths overflow";
                        return false;
                    }
                    while (rep--) len[i++] = val;
                }
            }
            Huffman lit, dist;
            if (!lit.build(len, hlit) || !dist.build(len + hlit, hdist) ||
                !inflate_block(br, lit, dist, out)) {
                err = "corrupt dynamic-Huffman block";
                return false;
            }
        } else {
            err = "reserved block type";
            return false;
        }
    }
    if (br.bad) {
        err = "truncated deflate stream";
        return false;
    }
    return true;
}

uint32_t be32(const uint8_t* p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    return (uint8_t)(pa <= pb && pa <= pc ? a : (pb <= pc ? b : c));
}

} // namespace

bool decode_png(const uint8_t* data, size_t size, std::vector<uint8_t>& rgba, uint32_t& width,
                uint32_t& height, std::string& err) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (size < 8 || std::memcmp(data, sig, 8) != 0) {
        err = "not a PNG file";
        return false;
    }
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, palette, trns;
    size_t at = 8;
    bool have_ihdr = false;
    while (at + 12 <= size) {
        const uint32_t len = be32(data + at);
        const uint8_t* type = data + at + 4;
        if (at + 12 + (size_t)len > size) {
            err = "truncated chunk";
            return false;
        }
        const uint8_t* body = data + at + 8;
        if (!std::memcmp(type, "IHDR", 4) && len >= 13) {
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            have_ihdr = true;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            palette.assign(body, body + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        at += 12 + (size_t)len;
    }
    if (!have_ihdr || w == 0 || h == 0 || w > 32768 || h > 32768) {
        err = "missing or bad IHDR";
        return false;
    }
    if (interlace) {
        err = "interlaced PNG is not supported";
        return false;
    }
    int channels;
    switch (ctype) {
    case 0: channels = 1; break;
    case 2: channels = 3; break;
    case 3: channels = 1; break;
    case 4: channels = 2; break;
    case 6: channels = 4; break;
    default: err = "bad colour type"; return false;
    }
    const bool ok_depth = ctype == 3 ? (depth == 1 || depth == 2 || depth == 4 || depth == 8)
                                     : (depth == 8 || depth == 16);
    if (!ok_depth) {
        err = "unsupported bit depth " + std::to_string(depth);
        return false;
    }
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (w * channels * depth / 8 + 1));
    if (!inflate_zlib(idat.data(), idat.size(), raw, err)) return false;
    const size_t stride = ((size_t)w * channels * depth + 7) / 8;
    if (raw.size() < (stride + 1) * h) {
        err = "image data too short";
        return false;
    }
    const int bpp = std::max(1, channels * depth / 8);
    std::vector<uint8_t> prev(stride, 0), cur(stride);
    rgba.assign((size_t)w * h * 4, 0);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* line = raw.data() + (stride + 1) * y;
        const uint8_t f = line[0];
        for (size_t x = 0; x < stride; ++x) {
            const int a = x >= (size_t)bpp ? cur[x - bpp] : 0, b = prev[x],
                      c = x >= (size_t)bpp ? prev[x - bpp] : 0;
            uint8_t v = line[1 + x];
            switch (f) {
            case 0: break;
            case 1: v = (uint8_t)(v + a); break;
            case 2: v = (uint8_t)(v + b); break;
            case 3: v = (uint8_t)(v + ((a + b) >> 1)); break;
            case 4: v = (uint8_t)(v + paeth(a, b, c)); break;
            default: err = "bad filter type"; return false;
            }
            cur[x] = v;
        }
        uint8_t* o = rgba.data() + (size_t)y * w * 4;
        for (uint32_t x = 0; x < w; ++x) {
            uint8_t px[4] = {0, 0, 0, 255};
            if (ctype == 3) {
                const int per = 8 / depth;
                const uint32_t byte = cur[x / per];
                const int shift = 8 - depth * (int)(x % per + 1);
                const uint32_t idx = (byte >> shift) & ((1u << depth) - 1u);
                if (3 * idx + 2 < palette.size()) {
                    px[0] = palette[3 * idx];
                    px[1] = palette[3 * idx + 1];
                    px[2] = palette[3 * idx + 2];
                }
                if (idx < trns.size()) px[3] = trns[idx];
            } else {
                const int bs = depth / 8; // bytes per sample (1 or 2, high byte first)
                auto sample = [&](int c) { return cur[((size_t)x * channels + c) * bs]; };
                if (ctype == 0 || ctype == 4) {
                    px[0] = px[1] = px[2] = sample(0);
                    if (ctype == 4) px[3] = sample(1);
                } else {
                    px[0] = sample(0);
                    px[1] = sample(1);
                    px[2] = sample(2);
                    if (ctype == 6) px[3] = sample(3);
                }
            }
            std::memcpy(o + 4 * x, px, 4);
        }
        std::swap(prev, cur);
    }
    width = w;
    height = h;
    return true;
}

bool read_png_file(const std::string& path, std::vector<uint8_t>& rgba, uint32_t& width,
                   uint32_t& height, std::string& err) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<uint8_t> data;
    uint8_t buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + got);
    std::fclose(f);
    return decode_png(data.data(), data.size(), rgba, width, height, err);
}

} // namespace gbpt

extern "C" GBPT_API int gbpt_image_read_png(const char* path, uint8_t* rgba, uint32_t* width,
                                            uint32_t* height) {
    if (!path || !width || !height) {
        gbpt::set_error("gbpt_image_read_png: null argument");
        return GBPT_ERR_INVALID;
    }
    std::vector<uint8_t> px;
    uint32_t w = 0, h = 0;
    std::string err;
    if (!gbpt::read_png_file(path, px, w, h, err)) {
        gbpt::set_error("gbpt_image_read_png: " + err);
        return GBPT_ERR_INVALID;
    }
    *width = w;
    *height = h;
    if (rgba) std::memcpy(rgba, px.data(), px.size());
    return GBPT_OK;
}

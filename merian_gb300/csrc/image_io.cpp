// PFM files, the float image format of merian's Image Write / Image Read nodes
// (src/merian/io/image_io.cpp:53-176): an ASCII header "PF" (3 channels) or "Pf" (1 channel),
// "width height", a scale whose sign gives the byte order (negative: little endian), then
// float32 scanlines from the bottom row up. RGBA input is written as RGB.
#include "context.h"
#include "gbpt.h"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace gbpt;

namespace {

uint32_t bswap32(uint32_t x) {
    return ((x & 0x000000FFu) << 24) | ((x & 0x0000FF00u) << 8) | ((x & 0x00FF0000u) >> 8) |
           ((x & 0xFF000000u) >> 24);
}

bool host_little_endian() {
    const uint32_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

} // namespace

extern "C" {

GBPT_API int gbpt_image_write_pfm(const char* path, const float* texels, uint32_t width,
                                  uint32_t height, uint32_t channels) {
    if (!path || !texels || width == 0 || height == 0 ||
        (channels != 1 && channels != 3 && channels != 4)) {
        set_error("gbpt_image_write_pfm: null argument, empty image or channels not 1, 3 or 4");
        return GBPT_ERR_INVALID;
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("gbpt_image_write_pfm: cannot open ") + path);
        return GBPT_ERR_INVALID;
    }
    const uint32_t out_c = channels == 1 ? 1 : 3;
    const bool le = host_little_endian();
    std::fprintf(f, "%s\n%u %u\n%s\n", out_c == 3 ? "PF" : "Pf", width, height, le ? "-1" : "1");
    std::vector<float> row((size_t)width * out_c);
    bool ok = true;
    for (uint32_t y = height; y-- > 0 && ok;) {
        const float* src = texels + (size_t)y * width * channels;
        for (uint32_t x = 0; x < width; ++x)
            for (uint32_t c = 0; c < out_c; ++c) row[(size_t)x * out_c + c] = src[(size_t)x * channels + c];
        ok = std::fwrite(row.data(), sizeof(float), row.size(), f) == row.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("gbpt_image_write_pfm: write failed for ") + path);
        return GBPT_ERR_INVALID;
    }
    return GBPT_OK;
}

// Reads a PFM into `texels` (top row first) with `channels` channels (1, 3 or 4; a missing
// channel repeats red, a missing alpha is 1). With texels == NULL only the size is returned.
GBPT_API int gbpt_image_read_pfm(const char* path, float* texels, uint32_t channels,
                                 uint32_t* width, uint32_t* height) {
    if (!path || !width || !height || (channels != 1 && channels != 3 && channels != 4)) {
        set_error("gbpt_image_read_pfm: null argument or channels not 1, 3 or 4");
        return GBPT_ERR_INVALID;
    }
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("gbpt_image_read_pfm: cannot open ") + path);
        return GBPT_ERR_NOT_FOUND;
    }
    char magic[3] = {0, 0, 0};
    unsigned w = 0, h = 0;
    float scale = 0.f;
    const bool header = std::fscanf(f, "%2s %u %u %f", magic, &w, &h, &scale) == 4;
    const int src_c = std::strcmp(magic, "PF") == 0 ? 3 : std::strcmp(magic, "Pf") == 0 ? 1 : 0;
    if (!header || src_c == 0 || w == 0 || h == 0 || scale == 0.f || std::fgetc(f) == EOF) {
        std::fclose(f);
        set_error(std::string("gbpt_image_read_pfm: malformed header in ") + path);
        return GBPT_ERR_INVALID;
    }
    *width = w;
    *height = h;
    if (!texels) {
        std::fclose(f);
        return GBPT_OK;
    }
    const bool swap = (scale < 0.f) != host_little_endian();
    std::vector<float> row((size_t)w * src_c);
    for (unsigned yf = 0; yf < h; ++yf) {
        if (std::fread(row.data(), sizeof(float), row.size(), f) != row.size()) {
            std::fclose(f);
            set_error(std::string("gbpt_image_read_pfm: truncated file ") + path);
            return GBPT_ERR_INVALID;
        }
        if (swap)
            for (float& v : row) {
                uint32_t b;
                std::memcpy(&b, &v, 4);
                b = bswap32(b);
                std::memcpy(&v, &b, 4);
            }
        float* dst = texels + (size_t)(h - 1 - yf) * w * channels;
        for (unsigned x = 0; x < w; ++x) {
            const float r = row[(size_t)x * src_c];
            const float g = src_c == 3 ? row[(size_t)x * src_c + 1] : r;
            const float b = src_c == 3 ? row[(size_t)x * src_c + 2] : r;
            float* px = dst + (size_t)x * channels;
            px[0] = r;
            if (channels >= 3) {
                px[1] = g;
                px[2] = b;
            }
            if (channels == 4) px[3] = 1.0f;
        }
    }
    std::fclose(f);
    return GBPT_OK;
}

} // extern "C"

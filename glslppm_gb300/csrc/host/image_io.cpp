// Image files for the resolved images of sppm_read_image (row 0 = the bottom row, as GL reads it).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "scene_internal.h"

namespace {

// little-endian byte writers (independent of the host's byte order)
struct Bytes {
    std::vector<unsigned char> b;
    void u8(unsigned v) { b.push_back((unsigned char)v); }
    void u32(uint32_t v) {
        for (int k = 0; k < 4; k++) u8((v >> (8 * k)) & 0xFFu);
    }
    void u64(uint64_t v) {
        for (int k = 0; k < 8; k++) u8((unsigned)((v >> (8 * k)) & 0xFFu));
    }
    void f32(float v) {
        uint32_t u;
        memcpy(&u, &v, 4);
        u32(u);
    }
    void str(const char* s) {  // with its terminating null
        do u8((unsigned char)*s); while (*s++);
    }
    // attribute: name, type name, byte size of the value (the value follows)
    void attr(const char* name, const char* type, uint32_t size) {
        str(name);
        str(type);
        u32(size);
    }
};

// OpenEXR 2 (the format's published layout): magic 20000630, version 2 with no flags (single-part
// scanline); the header's attributes, a null byte; one 64-bit file offset per scanline block; the
// blocks (one scanline each without compression): y, byte count, then each channel's row in the
// channel list's (alphabetical) order.  Rows run top to bottom.
bool write_exr(FILE* f, const float* rgb, uint32_t width, uint32_t height) {
    Bytes h;
    h.u32(20000630u);
    h.u32(2u);
    h.attr("channels", "chlist", 3 * (2 + 16) + 1);
    for (const char* name : {"B", "G", "R"}) {
        h.str(name);
        h.u32(2u);                // FLOAT
        h.u8(0);                  // pLinear
        h.u8(0), h.u8(0), h.u8(0);  // reserved
        h.u32(1u);                // x sampling
        h.u32(1u);                // y sampling
    }
    h.u8(0);
    h.attr("compression", "compression", 1);
    h.u8(0);  // NO_COMPRESSION
    for (const char* name : {"dataWindow", "displayWindow"}) {
        h.attr(name, "box2i", 16);
        h.u32(0u), h.u32(0u), h.u32(width - 1), h.u32(height - 1);
    }
    h.attr("lineOrder", "lineOrder", 1);
    h.u8(0);  // INCREASING_Y
    h.attr("pixelAspectRatio", "float", 4);
    h.f32(1.0f);
    h.attr("screenWindowCenter", "v2f", 8);
    h.f32(0.0f), h.f32(0.0f);
    h.attr("screenWindowWidth", "float", 4);
    h.f32(1.0f);
    h.u8(0);  // end of header
    const uint64_t block = 8 + (uint64_t)width * 12;
    const uint64_t first = h.b.size() + 8ull * height;
    for (uint32_t y = 0; y < height; y++) h.u64(first + y * block);
    if (fwrite(h.b.data(), 1, h.b.size(), f) != h.b.size()) return false;
    Bytes row;
    for (uint32_t y = 0; y < height; y++) {
        row.b.clear();
        row.u32(y);
        row.u32(width * 12u);
        const float* src = rgb + (size_t)(height - 1 - y) * width * 3;  // row 0 of rgb is the bottom
        for (int c = 2; c >= 0; c--)                                    // B, G, R
            for (uint32_t x = 0; x < width; x++) row.f32(src[(size_t)x * 3 + c]);
        if (fwrite(row.b.data(), 1, row.b.size(), f) != row.b.size()) return false;
    }
    return true;
}

}  // namespace

extern "C" int sppm_write_image_file(const char* path, const float* rgb, uint32_t width, uint32_t height,
                                     uint32_t format) {
    if (!path || !rgb) return sppm::fail(SPPM_ERR_ARG, "null argument");
    if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 30))
        return sppm::fail(SPPM_ERR_ARG, "image size %ux%u out of range", width, height);
    if (format != SPPM_FILE_PFM && format != SPPM_FILE_PPM && format != SPPM_FILE_EXR)
        return sppm::fail(SPPM_ERR_ARG, "unknown format %u", format);
    FILE* f = fopen(path, "wb");
    if (!f) return sppm::fail(SPPM_ERR_IO, "cannot open %s for writing", path);
    bool ok = true;
    const size_t row = (size_t)width * 3;
    if (format == SPPM_FILE_PFM) {
        // "PF", size, negative scale = little-endian floats; rows stored bottom to top
        ok = fprintf(f, "PF\n%u %u\n-1.0\n", width, height) > 0;
        uint16_t probe = 1;
        const bool little = *reinterpret_cast<uint8_t*>(&probe) == 1;
        std::vector<float> buf(row);
        for (uint32_t y = 0; ok && y < height; y++) {
            memcpy(buf.data(), rgb + y * row, row * sizeof(float));
            if (!little)
                for (auto& v : buf) {
                    uint32_t u;
                    memcpy(&u, &v, 4);
                    u = (u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24);
                    memcpy(&v, &u, 4);
                }
            ok = fwrite(buf.data(), sizeof(float), row, f) == row;
        }
    } else if (format == SPPM_FILE_EXR) {
        ok = write_exr(f, rgb, width, height);
    } else {
        // binary P6, top row first, 8 bits: clamp(v, 0, 1) * 255 rounded
        ok = fprintf(f, "P6\n%u %u\n255\n", width, height) > 0;
        std::vector<unsigned char> buf(row);
        for (uint32_t y = 0; ok && y < height; y++) {
            const float* src = rgb + (size_t)(height - 1 - y) * row;
            for (size_t i = 0; i < row; i++) {
                const float v = src[i] != src[i] ? 0.0f : std::fmin(std::fmax(src[i], 0.0f), 1.0f);
                buf[i] = (unsigned char)std::lround(v * 255.0f);
            }
            ok = fwrite(buf.data(), 1, row, f) == row;
        }
    }
    if (fclose(f) != 0) ok = false;
    if (!ok) return sppm::fail(SPPM_ERR_IO, "writing %s failed", path);
    return SPPM_OK;
}

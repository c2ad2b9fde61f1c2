// Image files for the resolved images of sppm_read_image (row 0 = the bottom row, as GL reads it).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "scene_internal.h"

extern "C" int sppm_write_image_file(const char* path, const float* rgb, uint32_t width, uint32_t height,
                                     uint32_t format) {
    if (!path || !rgb) return sppm::fail(SPPM_ERR_ARG, "null argument");
    if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 30))
        return sppm::fail(SPPM_ERR_ARG, "image size %ux%u out of range", width, height);
    if (format != SPPM_FILE_PFM && format != SPPM_FILE_PPM) return sppm::fail(SPPM_ERR_ARG, "unknown format %u", format);
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

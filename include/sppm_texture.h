/*
 * sppm_texture.h -- the reference's material textures (VolumeTextureTextures, gpurt.cpp:158-198)
 * and their sampling, shared by the CUDA kernels and the CPU restatement of the shader path.
 *
 * The reference resamples every material's map_Kd image to 512 x 512 (nearest texel: source
 * column x * w / 512, row y * h / 512, integer division) into one RGB8 3-D texture whose layer z is
 * material z; an untextured material's layer is magenta (255, 0, 255).  The shaders sample it with
 * GL_LINEAR filtering and GL_REPEAT wrapping in all three coordinates: at
 * (tex, (material + 0.5) / materials) on the eye path (eyeraytrace.fs:443-446) and at
 * (tex, (material + 0.75) / materials) for photon emission and bounces (photontrace.fs:418-422,
 * 562-565), so a photon's colour takes a quarter of the next material's layer.
 *
 * GL leaves the precision of linear filtering to the implementation; it is pinned here in IEEE
 * single precision with a fixed order of operations (the same on the host and the device):
 *   u = s * W - 0.5, i0 = floor(u), a = u - i0, i1 = i0 + 1, both wrapped into [0, W);
 *   the same for t (H, b) and r (D = number of materials, c);
 *   texels as byte / 255; lerp(p, q, f) = p * (1 - f) + q * f along x, then y, then z.
 * Layers are stored only for textured materials (layer_of_material[m] >= 0); other layers read
 * as magenta.
 */
#ifndef SPPM_TEXTURE_H
#define SPPM_TEXTURE_H

#include "sppm_fpmath.h"

#define SPPM_TEXTURE_RES 512

/* i mod n for an integral float i (GL_REPEAT), as an index in [0, n) */
SPPM_FP_FN int sppm_tex_wrap(float i, float n) {
    float w = sppm_sub(i, sppm_mul(n, floorf(sppm_div(i, n))));
    if (w < 0.0f) w = sppm_add(w, n);
    if (w >= n) w = sppm_sub(w, n);
    if (!(w >= 0.0f)) w = 0.0f; /* NaN coordinates read texel 0 */
    return (int)w;
}

SPPM_FP_FN float sppm_tex_lerp(float p, float q, float f) {
    return sppm_add(sppm_mul(p, sppm_sub(1.0f, f)), sppm_mul(q, f));
}

/* channel ch of texel (x, y) of material layer z: texels[layer][y][x][4] (RGBA8, A unused) */
SPPM_FP_FN float sppm_tex_texel(const uint8_t* texels, const int32_t* layer_of_material, int x, int y, int z, int ch) {
    const int32_t layer = layer_of_material[z];
    if (layer < 0) return ch == 1 ? 0.0f : 1.0f; /* magenta: 255 / 255, 0, 255 / 255 */
    const size_t i = (((size_t)layer * SPPM_TEXTURE_RES + (size_t)y) * SPPM_TEXTURE_RES + (size_t)x) * 4 + (size_t)ch;
    return sppm_div((float)texels[i], 255.0f);
}

/* texture3D(VolumeTextureTextures, (s, t, r)).rgb */
SPPM_FP_FN void sppm_tex_sample(const uint8_t* texels, const int32_t* layer_of_material, uint32_t num_materials,
                                float s, float t, float r, float out[3]) {
    const float W = (float)SPPM_TEXTURE_RES, D = (float)num_materials;
    const float u = sppm_sub(sppm_mul(s, W), 0.5f), v = sppm_sub(sppm_mul(t, W), 0.5f), w = sppm_sub(sppm_mul(r, D), 0.5f);
    const float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    const float a = sppm_sub(u, fu), b = sppm_sub(v, fv), c = sppm_sub(w, fw);
    const int x0 = sppm_tex_wrap(fu, W), x1 = sppm_tex_wrap(sppm_add(fu, 1.0f), W);
    const int y0 = sppm_tex_wrap(fv, W), y1 = sppm_tex_wrap(sppm_add(fv, 1.0f), W);
    const int z0 = sppm_tex_wrap(fw, D), z1 = sppm_tex_wrap(sppm_add(fw, 1.0f), D);
    for (int ch = 0; ch < 3; ch++) {
        const float c00 = sppm_tex_lerp(sppm_tex_texel(texels, layer_of_material, x0, y0, z0, ch),
                                        sppm_tex_texel(texels, layer_of_material, x1, y0, z0, ch), a);
        const float c10 = sppm_tex_lerp(sppm_tex_texel(texels, layer_of_material, x0, y1, z0, ch),
                                        sppm_tex_texel(texels, layer_of_material, x1, y1, z0, ch), a);
        const float c01 = sppm_tex_lerp(sppm_tex_texel(texels, layer_of_material, x0, y0, z1, ch),
                                        sppm_tex_texel(texels, layer_of_material, x1, y0, z1, ch), a);
        const float c11 = sppm_tex_lerp(sppm_tex_texel(texels, layer_of_material, x0, y1, z1, ch),
                                        sppm_tex_texel(texels, layer_of_material, x1, y1, z1, ch), a);
        out[ch] = sppm_tex_lerp(sppm_tex_lerp(c00, c10, b), sppm_tex_lerp(c01, c11, b), c);
    }
}

/* the reference's resampling of a w x h RGB8 image to the 512 x 512 layer (RGBA8, A = 255) */
static inline void sppm_tex_resample(const uint8_t* rgb, int w, int h, uint8_t* layer) {
    for (int y = 0; y < SPPM_TEXTURE_RES; y++)
        for (int x = 0; x < SPPM_TEXTURE_RES; x++) {
            const size_t src = 3 * ((size_t)(x * w / SPPM_TEXTURE_RES) + (size_t)(y * h / SPPM_TEXTURE_RES) * (size_t)w);
            uint8_t* d = layer + ((size_t)y * SPPM_TEXTURE_RES + (size_t)x) * 4;
            d[0] = rgb[src];
            d[1] = rgb[src + 1];
            d[2] = rgb[src + 2];
            d[3] = 255;
        }
}

#endif /* SPPM_TEXTURE_H */

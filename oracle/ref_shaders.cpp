// ref_shaders.cpp -- the reference's own GLSL shaders, compiled as C++ through glsl_compat.hpp and
// driven frame by frame the way m_display (glslppm.cpp:214-536) drives them through OpenGL.
//
// TEST INFRASTRUCTURE ONLY: it pins the C restatement (sppm_oracle.c) against the reference's shader
// sources.  The shader bodies are the reference files with the "#version" line removed and "f"
// appended to floating literals (oracle/build.py writes them into oracle/_ref, never into the
// repository); each is placed in its own namespace below.
//
// What OpenGL does between the draws is restated here:
//   * texture packing of CGPURT::CreateTextures (gpurt.cpp:47-552): six texels per triangle in a
//     square RGBA32F texture, two texels per material, the light CDF table, the 2X x 4Y BVH texture
//     (six hit/miss blocks, one min and one max block), the root-selecting cube map;
//   * full-screen quads: one fragment per texel, gl_FragCoord at the pixel centre, gl_TexCoord[0]
//     = (i + 0.5)/N * s (drawQuad / drawQuadwithTex);
//   * ReduceTexture's 2x2 ping-pong (glslppm.cpp:170-209) and its final texel read;
//   * GL_POINTS of the photon VBO (glslppm.cpp:784-795): clipping to the unit cube, a one-pixel
//     point at floor of the window coordinate, the GL_LESS depth test against a depth buffer
//     cleared to 1 (scatter), additive blending of 1.0 (correction);
//   * the uniforms and the host arithmetic of m_display.
// Scenes must be square, power-of-two sized (ImageResolution = PhotonBufferSize = HashResolution),
// untextured, as in the reference.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "glsl_compat.hpp"
#include "sppm.h"
#include "sppm_texture.h"

namespace glsl {
struct InOut {
    typedef ::glsl::vec2& vec2;
    typedef ::glsl::vec3& vec3;
    typedef ::glsl::vec4& vec4;
};
// VolumeTextureTextures of the scene being run (set by ref_gl_run_frames): GL_LINEAR + GL_REPEAT
// as include/sppm_texture.h pins them
static int g_texture3d_calls = 0;
static const uint8_t* g_tex = nullptr;
static const int32_t* g_layer = nullptr;
static uint32_t g_layers_nm = 0;
vec4 texture3D(const sampler3D&, const vec3& c) {
    g_texture3d_calls++;
    float t[3];
    sppm_tex_sample(g_tex, g_layer, g_layers_nm, c.x, c.y, c.z, t);
    return vec4(t[0], t[1], t[2], 1.0f);
}
}  // namespace glsl

#define uniform
#define varying
#define inout InOut::
#define out InOut::
#define in
#define main shader_main
#define GLSL_BUILTINS          \
    vec4 gl_TexCoord[1];       \
    vec4 gl_FragCoord;         \
    vec4 gl_FragData[8];       \
    vec4 gl_FragColor;         \
    vec4 gl_Vertex;            \
    vec4 gl_Position;

namespace glsl {
namespace sh_eye {
GLSL_BUILTINS
#include "eyeraytrace_fs.inc"
}
namespace sh_photon {
GLSL_BUILTINS
#include "photontrace_fs.inc"
}
namespace sh_hash {
GLSL_BUILTINS
#include "hash_fs.inc"
}
namespace sh_scatter {
GLSL_BUILTINS
#include "scatter_vs.inc"
}
namespace sh_correction {
GLSL_BUILTINS
#include "correction_vs.inc"
}
namespace sh_progressive {
GLSL_BUILTINS
#include "progressive_fs.inc"
}
namespace sh_re {
GLSL_BUILTINS
#include "re_fs.inc"
}
namespace sh_min {
GLSL_BUILTINS
#include "min_fs.inc"
}
namespace sh_max {
GLSL_BUILTINS
#include "max_fs.inc"
}
namespace sh_sum {
GLSL_BUILTINS
#include "sum_fs.inc"
}
}  // namespace glsl

#undef uniform
#undef varying
#undef inout
#undef out
#undef in
#undef main

using namespace glsl;

namespace {

struct Tex {
    int w = 0, h = 0;
    std::vector<vec4> t;
    void init(int W, int H, vec4 v = vec4(0.0f)) {
        w = W;
        h = H;
        t.assign((size_t)W * H, v);
    }
    sampler2D s() const {
        sampler2D r;
        r.texels = t.data();
        r.w = w;
        r.h = h;
        return r;
    }
    vec4& at(int i, int j) { return t[(size_t)j * w + i]; }
};

struct XorShift {  // glslppm.cpp:77-91
    uint32_t x = 123456789u, y = 362436069u, z = 521288629u, w = 88675123u;
    float frand() {
        const uint32_t t = x ^ (x << 11);
        x = y;
        y = z;
        z = w;
        return (w = (w ^ (w >> 19)) ^ (t ^ (t >> 8))) * (1.0f / 4294967295.0f);
    }
};

struct RefGL {
    int R = 0;  // ImageResolution = PhotonBufferSize = HashResolution
    int max_bounces = 10;
    // scene textures
    Tex polys, mats, lights, bvh;
    samplerCube roots;
    int poly_x = 0, bbox_x = 0, bbox_y = 0;
    float poly_stride[2] = {0, 0}, material_stride = 0, light_stride = 0, light_area = 0, material_num_rcp = 0;
    int num_lights = 0;
    vec4 scene_bsphere;
    // VolumeTextureTextures: the textured materials' 512x512 layers, the others magenta
    std::vector<uint8_t> tex;
    std::vector<int32_t> mat_layer;
    // state textures
    Tex q_pos, q_refl, q_nrm, rnd_eye, q_isect, q_emi, q_flux;
    Tex p_pos, p_flux, p_dir, rnd_photon, p_isect, p_emitted, p_index, p_hash, p_corr, minmax_q, minmax_p;
    std::vector<float> depth;
    // camera
    sppm_camera cam;
    XorShift xs;
    unsigned frame = 0, eye_samples = 0;
    float num_photons = 0.0f;
    vec4 bbmax, bbmin;
    float initial_radius = 0, grid_scale = 0;
    float focal = 13.0f, aperture = 0.0f;
};

template <class F>
void draw_quad(int n, float s_range, F&& frag) {
    // drawQuad / drawQuadwithTex: an n x n viewport, texcoords [0, s_range]
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            const vec2 tc(((float)i + 0.5f) / (float)n * s_range, ((float)j + 0.5f) / (float)n * s_range);
            frag(i, j, tc);
        }
}

// ---------------------------------------------------------------------------------------------
// CGPURT::CreateTextures (gpurt.cpp:47-552)
// ---------------------------------------------------------------------------------------------
void create_textures(RefGL& g, const sppm_scene* s) {
    const int nt = (int)s->num_triangles;
    std::vector<vec2> tri_tc(nt);
    const int X = int(sqrtf(nt * 6.0f) + 1.0f);
    g.poly_x = X;
    g.poly_stride[0] = 1.0f / float(X);
    g.poly_stride[1] = 1.0f / float(X);
    g.polys.init(X, X);
    for (int k = 0; k < nt * 6; k += 6) {
        const int p = k / 6;
        const int i = k % X, j = k / X;
        tri_tc[p] = vec2(((float)i + 0.5f) / (float)X, ((float)j + 0.5f) / (float)X);
        for (int v = 0; v < 3; v++) {
            const float* pos = s->positions + (size_t)p * 9 + v * 3;
            const float tu = s->texcoords ? s->texcoords[p * 6 + v * 2] : 1.0e30f;
            g.polys.t[k + v] = vec4(pos[0], pos[1], pos[2], tu);
        }
        for (int v = 0; v < 3; v++) {
            const float* n = s->normals + (size_t)p * 9 + v * 3;
            const float tv = s->texcoords ? s->texcoords[p * 6 + v * 2 + 1] : 1.0e30f;
            const float sg = n[2] > 0.0f ? 1.0f : -1.0f;
            g.polys.t[k + 3 + v] = vec4(n[0], n[1], sg * (float)(s->material_ids[p] + 1), tv);
        }
    }
    const int nm = (int)s->num_materials;
    g.material_stride = 1.0f / (float)nm;
    g.material_num_rcp = 1.0f / float(nm);
    g.mats.init(nm * 2, 1);
    for (int m = 0; m < nm; m++) {
        const sppm_material& mm = s->materials[m];
        g.mats.t[m * 2] = vec4(mm.color[0], mm.color[1], mm.color[2], mm.eta);
        g.mats.t[m * 2 + 1] = vec4((float)mm.brdf, mm.glossiness, 0.0f, 0.0f);
    }
    g.num_lights = (int)s->num_lights;
    g.light_area = s->light_area;
    g.light_stride = g.num_lights ? 1.0f / (float)g.num_lights : 0.0f;
    g.lights.init(g.num_lights ? g.num_lights : 1, 1);
    for (int l = 0; l < g.num_lights; l++)
        g.lights.t[l] = vec4(tri_tc[s->light_triangles[l]].x, tri_tc[s->light_triangles[l]].y, s->light_cdf[l], 0.0f);
    // BVH texture
    const int nn = (int)s->num_nodes;
    const int BX = int(sqrtf(float(nn)) + 1.0f), BY = BX;
    g.bbox_x = BX;
    g.bbox_y = BY;
    for (int f = 0; f < 6; f++) {
        const float ox = (f & 1) ? 1.0f : 0.0f, oy = (float)(f / 2);
        g.roots.face[f] = vec4(((float)BX * ox + 0.5f) / ((float)BX * 2.0f), ((float)BY * oy + 0.5f) / ((float)BY * 4.0f),
                               -1.0f, -1.0f);
    }
    auto tc_of = [&](int kk, int k) {  // BBoxTexCoord[kk][k]
        const int offx = (kk & 1) ? BX : 0, offy = (kk / 2) * BY;
        const int i = k % BX, j = k / BX;
        return vec2((float)(i + offx + 0.5f) / ((float)BX * 2.0f), (float)(j + offy + 0.5f) / ((float)BY * 4.0f));
    };
    g.bvh.init(BX * 2, BY * 4);
    for (int kk = 0; kk < 6; kk++) {
        const int32_t* base = s->order_base + (size_t)kk * nn;
        const int32_t* miss = s->order_miss + (size_t)kk * nn;
        std::vector<int> pos_of(nn);
        for (int i = 0; i < nn; i++) pos_of[base[i]] = i;
        for (int c = 0; c < nn; c++) {
            const int i = pos_of[c];  // position of canonical node c in ordering kk
            const vec2 hit = (i + 1 >= nn) ? vec2(-1.0f, -1.0f) : tc_of(kk, base[i + 1]);
            const vec2 ms = (miss[i] == -1 || miss[i] >= nn) ? vec2(-1.0f, -1.0f) : tc_of(kk, base[miss[i]]);
            const int offx = (kk & 1) ? BX : 0, offy = (kk / 2) * BY;
            g.bvh.at(c % BX + offx, c / BX + offy) = vec4(hit.x, hit.y, ms.y, ms.x);
        }
    }
    for (int j = 0; j < BY; j++)
        for (int i = 0; i < BX; i++) {
            const int k = j * BX + i;
            vec4 mn(-1.0f, -1.0f, -1.0f, 0.0f), mx(1.0f, 1.0f, 1.0f, 0.0f);
            if (k < nn) {
                const float* b = s->node_bounds + (size_t)k * 6;
                const int tri = s->node_triangle[k];
                mn = vec4(b[0], b[1], b[2], tri != -1 ? tri_tc[tri].x : -1.0f);
                mx = vec4(b[3], b[4], b[5], tri != -1 ? tri_tc[tri].y : -1.0f);
            }
            g.bvh.at(i, j + 3 * BY) = mn;
            g.bvh.at(i + BX, j + 3 * BY) = mx;
        }
    const float* mn = s->bbox_min;
    const float* mx = s->bbox_max;
    const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    g.scene_bsphere = vec4((mx[0] + mn[0]) * 0.5f, (mx[1] + mn[1]) * 0.5f, (mx[2] + mn[2]) * 0.5f,
                           std::sqrt(dx * dx + dy * dy + dz * dz) * 0.5f);
}

// ReduceTexture (glslppm.cpp:170-209) with one of min.fs / max.fs / sum.fs
enum { RED_MIN, RED_MAX, RED_SUM };
vec4 reduce_texture(Tex& work, const Tex& src, int op) {
    const int R = src.w;
    auto run = [&](const Tex& in, float off, int n) {
        std::vector<vec4> outv((size_t)n * n);
        draw_quad(n, off, [&](int i, int j, vec2 tc) {
            vec4 r;
            switch (op) {
                case RED_MIN:
                    sh_min::Texture = in.s();
                    sh_min::Offset = vec2(off, off);
                    sh_min::gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
                    sh_min::shader_main();
                    r = sh_min::gl_FragColor;
                    break;
                case RED_MAX:
                    sh_max::Texture = in.s();
                    sh_max::Offset = vec2(off, off);
                    sh_max::gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
                    sh_max::shader_main();
                    r = sh_max::gl_FragColor;
                    break;
                default:
                    sh_sum::Texture = in.s();
                    sh_sum::Offset = vec2(off, off);
                    sh_sum::gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
                    sh_sum::shader_main();
                    r = sh_sum::gl_FragColor;
                    break;
            }
            outv[(size_t)j * n + i] = r;
        });
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) work.at(i, j) = outv[(size_t)j * n + i];
    };
    unsigned level = 1;
    unsigned reduced = R >> level;
    float off = 1.0f / float(1 << level);
    run(src, off, (int)reduced);
    const unsigned passes = (unsigned)(log((double)(R >> level)) / log(2.0)) + 1;
    vec4 result;
    for (unsigned p = 0; p < passes; p++) {
        level++;
        off = 1.0f / float(1 << level);
        reduced = R >> level;
        if (reduced) run(work, off, (int)reduced);
        result = work.at(0, 0);  // glReadPixels(0, 0, 1, 1)
    }
    return result;
}

void set_trace_uniforms_eye(RefGL& g) {
    using namespace sh_eye;
    const float bx = (float)g.bbox_x, by = (float)g.bbox_y;
    OffsetToBBoxMinMax = vec4(0.5f / (bx * 2.0f), (by * 3.0f + 0.5f) / (by * 4.0f), (bx + 0.5f) / (bx * 2.0f),
                              (by * 3.0f + 0.5f) / (by * 4.0f));
    TexturePolygons = g.polys.s();
    CubeTextureBBoxRootIndices = g.roots;
    TextureBVH = g.bvh.s();
    TextureMaterials = g.mats.s();
    MaterialStride = g.material_stride;
    MaterialNumRcp = g.material_num_rcp;
    LightSummedArea = g.light_area;
    CameraPosition = vec3(g.cam.origin[0], g.cam.origin[1], g.cam.origin[2]);
    CameraU = vec3(g.cam.u[0], g.cam.u[1], g.cam.u[2]);
    CameraV = vec3(g.cam.v[0], g.cam.v[1], g.cam.v[2]);
    CameraW = vec3(g.cam.w[0], g.cam.w[1], g.cam.w[2]);
    CameraParams = vec3((float)g.cam.width * 0.5f, (float)g.cam.height * 0.5f, g.cam.distance);
    FocalLength = g.focal;
    MaxPathLength = g.max_bounces;
    ApertureSize = g.aperture;
    PolygonDataStride = vec2(g.poly_stride[0], g.poly_stride[1]);
}

void run_frame(RefGL& g) {
    const int R = g.R;
    if (g.frame == 0)
        for (auto& v : g.q_emi.t) v = vec4(0.0f);
    if (g.frame % (unsigned)g.max_bounces == 0) {
        set_trace_uniforms_eye(g);
        const float ax = (g.xs.frand() - 0.5f) * 1.25f;
        const float ay = (g.xs.frand() - 0.5f) * 1.25f;
        sh_eye::AAOffset = vec2(ax, ay);
        sh_eye::RandomTexture = g.rnd_eye.s();
        sh_eye::QueryEmissionPhotonCountTexture = g.q_emi.s();
        sh_eye::NumEyeSamples = (int)g.eye_samples + 1;
        g.eye_samples++;
        std::vector<vec4> o[6];
        for (auto& v : o) v.resize((size_t)R * R);
        draw_quad(R, 1.0f, [&](int i, int j, vec2 tc) {
            sh_eye::gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
            sh_eye::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.5f, 1.0f);
            sh_eye::shader_main();
            for (int k = 0; k < 6; k++) o[k][(size_t)j * R + i] = sh_eye::gl_FragData[k];
        });
        g.q_pos.t = o[0];
        g.q_refl.t = o[1];
        g.q_nrm.t = o[2];
        g.rnd_eye.t = o[3];
        g.q_isect.t = o[4];
        g.q_emi.t = o[5];
        g.bbmax = reduce_texture(g.minmax_q, g.q_pos, RED_MAX);
        g.bbmin = reduce_texture(g.minmax_q, g.q_pos, RED_MIN);
        float bbsize = 0.0f;
        for (int i = 0; i < 3; i++) bbsize += g.bbmax[i] - g.bbmin[i];
        g.initial_radius = (bbsize / 3.0f) / (float)(R) * 2.5f;
        for (int i = 0; i < 3; i++) {
            g.bbmin[i] -= g.initial_radius;
            g.bbmax[i] += g.initial_radius;
        }
        g.grid_scale = 0.5f / g.initial_radius;
    }
    if (g.frame == 0) {
        for (auto& v : g.q_flux.t) v = vec4(0.0f, 0.0f, 0.0f, g.initial_radius);
        for (auto& v : g.p_isect.t) v = vec4(-1.0f, -1.0f, 0.0f, 1.0e+30f);
        g.num_photons = 0.0f;
    }
    {  // photon tracing
        using namespace sh_photon;
        const float bx = (float)g.bbox_x, by = (float)g.bbox_y;
        OffsetToBBoxMinMax = vec4(0.5f / (bx * 2.0f), (by * 3.0f + 0.5f) / (by * 4.0f), (bx + 0.5f) / (bx * 2.0f),
                                  (by * 3.0f + 0.5f) / (by * 4.0f));
        TexturePolygons = g.polys.s();
        CubeTextureBBoxRootIndices = g.roots;
        TextureBVH = g.bvh.s();
        PolygonDataStride = vec2(g.poly_stride[0], g.poly_stride[1]);
        PhotonIntersectionTexture = g.p_isect.s();
        PhotonPositionTexture = g.p_pos.s();
        PhotonFluxTexture = g.p_flux.s();
        PhotonDirectionTexture = g.p_dir.s();
        TextureMaterials = g.mats.s();
        MaterialStride = g.material_stride;
        MaterialNumRcp = g.material_num_rcp;
        TextureLightSources = g.lights.s();
        LightSourceStride = g.light_stride;
        LightSummedArea = g.light_area;
        RandomTexture = g.rnd_photon.s();
        MaxPathLength = g.max_bounces;
        SceneBSphere = g.scene_bsphere;
        std::vector<vec4> o[6];
        for (auto& v : o) v.resize((size_t)R * R);
        draw_quad(R, 1.0f, [&](int i, int j, vec2 tc) {
            gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
            gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.5f, 1.0f);
            shader_main();
            for (int k = 0; k < 6; k++) o[k][(size_t)j * R + i] = gl_FragData[k];
        });
        g.p_pos.t = o[0];
        g.p_flux.t = o[1];
        g.p_dir.t = o[2];
        g.rnd_photon.t = o[3];
        g.p_isect.t = o[4];
        g.p_emitted.t = o[5];
        const vec4 n = reduce_texture(g.minmax_p, g.p_emitted, RED_SUM);
        g.num_photons += int(n.x);
    }
    {  // hash keys
        using namespace sh_hash;
        BufInfo = vec4((float)R, (float)R, 1.0f / float(R), 1.0f / float(R));
        HashNum = R * R;
        GridScale = g.grid_scale;
        HashScale1 = 4194304.0f / g.grid_scale;
        BBoxMin = vec3(g.bbmin.x, g.bbmin.y, g.bbmin.z);
        PhotonPositionTexture = g.p_pos.s();
        PhotonFluxTexture = g.p_flux.s();
        std::vector<vec4> o((size_t)R * R);
        draw_quad(R, 1.0f, [&](int i, int j, vec2 tc) {
            gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
            shader_main();
            o[(size_t)j * R + i] = gl_FragColor;
        });
        g.p_index.t = o;
    }
    {  // scatter (GL_POINTS, GL_LESS depth test) and correction (additive blend)
        for (auto& v : g.p_hash.t) v = vec4(0.0f);
        for (auto& v : g.p_corr.t) v = vec4(0.0f);
        std::fill(g.depth.begin(), g.depth.end(), 1.0f);
        sh_scatter::BufInfo = vec4((float)R, (float)R, 1.0f / float(R), 1.0f / float(R));
        sh_scatter::PhotonIndexTexture = g.p_index.s();
        sh_scatter::PhotonBufferSize1 = 1.0f / float(R);
        sh_correction::BufInfo = sh_scatter::BufInfo;
        sh_correction::PhotonIndexTexture = g.p_index.s();
        for (int j = 0; j < R; j++)
            for (int i = 0; i < R; i++) {
                const vec4 vtx(2.0f * (((float)i + 0.5f) / float(R)) - 1.0f, 2.0f * (((float)j + 0.5f) / float(R)) - 1.0f,
                               0.0f, 1.0f);
                sh_scatter::gl_Vertex = vtx;
                sh_scatter::shader_main();
                const vec4 P = sh_scatter::gl_Position;
                if (P.x >= -1.0f && P.x <= 1.0f && P.y >= -1.0f && P.y <= 1.0f && P.z >= -1.0f && P.z <= 1.0f) {
                    const int px = (int)std::floor((P.x + 1.0f) * 0.5f * (float)R);
                    const int py = (int)std::floor((P.y + 1.0f) * 0.5f * (float)R);
                    const float zw = P.z * 0.5f + 0.5f;
                    if (px >= 0 && px < R && py >= 0 && py < R && zw < g.depth[(size_t)py * R + px]) {
                        g.depth[(size_t)py * R + px] = zw;
                        g.p_hash.at(px, py) = sh_scatter::p;  // scatter.fs: gl_FragColor = p
                    }
                }
                sh_correction::gl_Vertex = vtx;
                sh_correction::shader_main();
                const vec4 Q = sh_correction::gl_Position;
                if (Q.x >= -1.0f && Q.x <= 1.0f && Q.y >= -1.0f && Q.y <= 1.0f) {
                    const int px = (int)std::floor((Q.x + 1.0f) * 0.5f * (float)R);
                    const int py = (int)std::floor((Q.y + 1.0f) * 0.5f * (float)R);
                    if (px >= 0 && px < R && py >= 0 && py < R) g.p_corr.at(px, py) = g.p_corr.at(px, py) + vec4(1.0f);
                }
            }
    }
    {  // progressive update
        using namespace sh_progressive;
        HashMax = vec3(std::fabs(g.bbmax[0] + g.initial_radius - g.bbmin[0]) * g.grid_scale,
                       std::fabs(g.bbmax[1] + g.initial_radius - g.bbmin[1]) * g.grid_scale,
                       std::fabs(g.bbmax[2] + g.initial_radius - g.bbmin[2]) * g.grid_scale);
        BufInfo = vec4((float)R, (float)R, 1.0f / float(R), 1.0f / float(R));
        HashNum = (float)(R * R);
        GridScale = g.grid_scale;
        HashScale1 = 4194304.0f / g.grid_scale;
        Alpha = 0.7f;
        BBoxMin = vec3(g.bbmin.x, g.bbmin.y, g.bbmin.z);
        HashedPhotonTexture = g.p_hash.s();
        PhotonCorrectionTexture = g.p_corr.s();
        QueryNormalTexture = g.q_nrm.s();
        QueryPositionTexture = g.q_pos.s();
        QueryEmissionPhotonCountTexture = g.q_emi.s();
        QueryFluxRadiusTexture = g.q_flux.s();
        QueryReflectanceTexture = g.q_refl.s();
        PhotonFluxTexture = g.p_flux.s();
        PhotonPositionTexture = g.p_pos.s();
        PhotonDirectionTexture = g.p_dir.s();
        QueryIntersectionTexture = g.q_isect.s();
        std::vector<vec4> o0((size_t)R * R), o1((size_t)R * R);
        draw_quad(R, 1.0f, [&](int i, int j, vec2 tc) {
            gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
            Flux = vec3(0.0f);  // the shader's global accumulators start at zero for each fragment
            PhotonCount = 0.0f;
            shader_main();
            o0[(size_t)j * R + i] = gl_FragData[0];
            o1[(size_t)j * R + i] = gl_FragData[1];
        });
        g.q_flux.t = o0;
        g.q_emi.t = o1;
    }
    g.frame++;
}

}  // namespace

#define EXPORT extern "C" __attribute__((visibility("default")))

EXPORT void* ref_gl_create(const sppm_scene* scene, const sppm_camera* cam, int resolution) {
    RefGL* g = new RefGL();
    glsl::g_texture3d_calls = 0;  // lookups are counted per harness
    g->R = resolution;
    g->cam = *cam;
    create_textures(*g, scene);
    g->mat_layer.assign(scene->num_materials, -1);
    if (scene->num_textures && scene->textures && scene->material_texture) {
        g->mat_layer.assign(scene->material_texture, scene->material_texture + scene->num_materials);
        g->tex.assign(scene->textures, scene->textures + (size_t)scene->num_textures * SPPM_TEXTURE_RES *
                                                            SPPM_TEXTURE_RES * 4);
    }
    const int R = resolution;
    for (Tex* t : {&g->q_pos, &g->q_refl, &g->q_nrm, &g->rnd_eye, &g->q_isect, &g->q_emi, &g->q_flux, &g->p_pos,
                   &g->p_flux, &g->p_dir, &g->rnd_photon, &g->p_isect, &g->p_emitted, &g->p_index, &g->p_hash,
                   &g->p_corr, &g->minmax_q, &g->minmax_p})
        t->init(R, R);
    g->depth.assign((size_t)R * R, 1.0f);
    // RandomizeTextures (glslppm.cpp:113-140): the four frand() calls are the arguments of one
    // TVector4 constructor call, an order C++ leaves unspecified; g++ (the reference's compiler)
    // evaluates them right to left, so the w lane receives the first draw
    for (Tex* t : {&g->rnd_eye, &g->rnd_photon})
        for (auto& v : t->t) {
            const float w = (float)(g->xs.frand() * 4194304.0), z = (float)(g->xs.frand() * 4194304.0);
            const float y = (float)(g->xs.frand() * 4194304.0), x = (float)(g->xs.frand() * 4194304.0);
            v = vec4(x, y, z, w);
        }
    return g;
}

// FocalLength / ApertureSize (glslppm.cpp:31-32, keyboard-adjustable in the reference)
EXPORT void ref_gl_set_lens(void* h, float focal, float aperture) {
    RefGL* g = (RefGL*)h;
    g->focal = focal;
    g->aperture = aperture;
}

EXPORT int ref_gl_run_frames(void* h, unsigned n) {
    RefGL* g = (RefGL*)h;
    glsl::g_tex = g->tex.empty() ? nullptr : g->tex.data();
    glsl::g_layer = g->mat_layer.data();
    glsl::g_layers_nm = (uint32_t)g->mat_layer.size();
    for (unsigned k = 0; k < n; k++) run_frame(*g);
    return glsl::g_texture3d_calls;
}

// texture by name: 0 QueryPosition, 1 QueryReflectance, 2 QueryNormal, 3 RandomEye, 4 QueryIntersection,
// 5 QueryEmissionPhotonCount, 6 QueryFluxRadius, 7 PhotonPosition, 8 PhotonFlux, 9 PhotonDirection,
// 10 RandomPhoton, 11 PhotonIntersection, 12 PhotonHash, 13 PhotonCorrection, 14 PhotonIndex
EXPORT int ref_gl_read(void* h, int which, float* dst) {
    RefGL* g = (RefGL*)h;
    Tex* t[] = {&g->q_pos, &g->q_refl, &g->q_nrm, &g->rnd_eye, &g->q_isect, &g->q_emi, &g->q_flux, &g->p_pos,
                &g->p_flux, &g->p_dir, &g->rnd_photon, &g->p_isect, &g->p_hash, &g->p_corr, &g->p_index};
    if (which < 0 || which > 14) return -1;
    for (size_t i = 0; i < t[which]->t.size(); i++)
        for (int c = 0; c < 4; c++) dst[i * 4 + c] = t[which]->t[i][c];
    return 0;
}

// scalars: frame, eye samples, NumPhotons, InitialRadius, GridScale, BBMin xyz, BBMax xyz,
// polygon texture width, image display from re.fs (rgb, written into dst + 16 when asked)
EXPORT void ref_gl_scalars(void* h, float* out) {
    RefGL* g = (RefGL*)h;
    out[0] = (float)g->frame;
    out[1] = (float)g->eye_samples;
    out[2] = g->num_photons;
    out[3] = g->initial_radius;
    out[4] = g->grid_scale;
    for (int i = 0; i < 3; i++) {
        out[5 + i] = g->bbmin[i];
        out[8 + i] = g->bbmax[i];
    }
    out[11] = (float)g->poly_x;
}

// re.fs over the image (display image, rgb per pixel)
EXPORT void ref_gl_display(void* h, float* rgb) {
    RefGL* g = (RefGL*)h;
    using namespace sh_re;
    TotalPhotonNum = g->num_photons;
    QueryEmissionPhotonCountTexture = g->q_emi.s();
    QueryFluxRadiusTexture = g->q_flux.s();
    const int R = g->R;
    draw_quad(R, 1.0f, [&](int i, int j, vec2 tc) {
        gl_TexCoord[0] = vec4(tc, 0.0f, 1.0f);
        shader_main();
        for (int c = 0; c < 3; c++) rgb[((size_t)j * R + i) * 3 + c] = gl_FragColor[c];
    });
}

EXPORT void ref_gl_destroy(void* h) { delete (RefGL*)h; }

// ReduceTexture with min.fs (op 0), max.fs (op 1) or sum.fs (op 2) on an R x R float4 texture
EXPORT void ref_gl_reduce(const float* texels, int R, int op, float* out) {
    Tex src, work;
    src.init(R, R);
    work.init(R, R);
    for (size_t i = 0; i < src.t.size(); i++) src.t[i] = vec4(texels[i * 4], texels[i * 4 + 1], texels[i * 4 + 2], texels[i * 4 + 3]);
    const vec4 r = reduce_texture(work, src, op == 0 ? RED_MIN : (op == 1 ? RED_MAX : RED_SUM));
    for (int c = 0; c < 4; c++) out[c] = r[c];
}

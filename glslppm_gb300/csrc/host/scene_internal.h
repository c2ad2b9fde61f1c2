// Host-side scene representation shared by the OBJ loader, the BVH builder and the device packer.
// All floating-point arithmetic in this directory is compiled with -ffp-contract=off so that
// every value is the IEEE single-precision result of the expression as written; the reference's
// host code (mesh.cpp, bvh.cpp, camera.cpp) performs the same operations in the same order, which
// the tests check against the reference compiled from its own sources.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "sppm.h"

namespace sppm {

struct V3 {
    float x, y, z;
};
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// cross product in the component order of vector.h:38 and of GLSL cross()
static inline V3 cross3(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
float sqrt_f32(float x);  // correctly rounded single-precision square root
// v * (1 / |v|), the form of vector.h:35 and of the pinned GLSL normalize()
static inline V3 normalize3(V3 v) { return v * (1.0f / sqrt_f32(dot3(v, v))); }

struct Box {
    V3 mn, mx;
    void init() {  // bbox.cpp:30-34
        mn = v3(1e+38f, 1e+38f, 1e+38f);
        mx = v3(-1e+38f, -1e+38f, -1e+38f);
    }
    void expand(V3 p) {  // bbox.cpp:24-28 (vector.h:39-40 select semantics)
        mx = v3(mx.x > p.x ? mx.x : p.x, mx.y > p.y ? mx.y : p.y, mx.z > p.z ? mx.z : p.z);
        mn = v3(mn.x < p.x ? mn.x : p.x, mn.y < p.y ? mn.y : p.y, mn.z < p.z ? mn.z : p.z);
    }
    float area() const {  // bbox.cpp:18-22
        const V3 l = mx - mn;
        return 2.0f * (l.x * l.y + l.y * l.z + l.z * l.x);
    }
};

}  // namespace sppm

struct sppm_mesh {
    uint32_t num_triangles = 0;
    std::vector<float> positions;  // [n][3][3]
    std::vector<float> normals;    // [n][3][3]
    std::vector<float> texcoords;  // [n][3][2]
    std::vector<int32_t> material_ids;
    std::vector<sppm_material> materials;
    std::vector<int32_t> light_triangles;
    std::vector<float> light_cdf;
    float light_area = 0.0f;
    sppm::Box bbox;
    std::vector<sppm::Box> tri_bbox;
    std::vector<sppm::V3> tri_centroid;
    // BVH (empty until sppm_mesh_build_bvh)
    uint32_t num_nodes = 0;
    std::vector<float> node_bounds;     // [num_nodes][6]
    std::vector<int32_t> node_triangle; // [num_nodes]
    std::vector<int32_t> order_base;    // [6][num_nodes]
    std::vector<int32_t> order_miss;    // [6][num_nodes]
    // material textures (map_Kd) resampled to 512x512 RGBA8; material_texture[m] = layer or -1
    std::vector<uint8_t> textures;
    std::vector<int32_t> material_texture;
    uint32_t num_textures = 0;

    sppm::V3 pos(uint32_t t, int v) const {
        const float* p = &positions[(size_t)t * 9 + v * 3];
        return sppm::v3(p[0], p[1], p[2]);
    }
    void finish_geometry();  // TMesh::CalculateBBox
    void prepare_lights();   // TMesh::PrepareLightSources
};

namespace sppm {
void set_error(const char* fmt, ...);
int fail(int status, const char* fmt, ...);
}  // namespace sppm

// TEST INFRASTRUCTURE: a stand-in for the reference's mesh.h with the members include/sppm_gpurt.hpp
// reads (TVector3, TBBox, TTriangle, TMaterial, TMesh), implemented over this library's own OBJ
// loader (sppm_mesh_load_obj).  It lets the drop-in header be compiled and rendered on machines
// that do not have the reference's sources; where they are present, the reference's own mesh.cpp
// is compiled instead (oracle/ref_gpurt_shim_test.cpp).
#pragma once

#include <cstdint>
#include <cstring>
#include <vector>

#include "sppm.h"

struct TVector3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    TVector3() = default;
    TVector3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
};

struct TBBox {
    TVector3 min, max;
};

struct TTriangle {
    TVector3 positions[3], normals[3], texcoords[3];
    int idMaterial = 0;
};

struct TMaterial {
    TVector3 color;
    float eta = 1.0f;
    int brdf = 0;
    float specularity = 0.0f;
    bool isTextured = false;
    int textureWidth = 0, textureHeight = 0;
    std::vector<unsigned char> texture;
};

class TMesh {
public:
    std::vector<TTriangle> triangles;
    std::vector<TMaterial> materials;
    std::vector<float> lightsCDF;
    std::vector<int> lightsIndices;
    float lightsArea = 0.0f;
    TBBox bbox;
    sppm_mesh* handle = nullptr;  // the library's mesh the members were read from

    ~TMesh() { Release(); }

    // reads the OBJ with the library's loader (the reference's parsing rules) and copies what
    // the reference's TMesh would hold
    bool LoadOBJ(const char* path, TVector3 offset, float scale) {
        Release();
        const float off[3] = {offset.x, offset.y, offset.z};
        if (sppm_mesh_load_obj(path, off, scale, &handle) != SPPM_OK) return false;
        sppm_scene s;
        if (sppm_mesh_get_scene(handle, &s) != SPPM_OK) return false;
        triangles.resize(s.num_triangles);
        for (uint32_t i = 0; i < s.num_triangles; i++) {
            TTriangle& t = triangles[i];
            for (int v = 0; v < 3; v++) {
                const float* p = s.positions + (size_t)i * 9 + v * 3;
                const float* n = s.normals + (size_t)i * 9 + v * 3;
                t.positions[v] = TVector3(p[0], p[1], p[2]);
                t.normals[v] = TVector3(n[0], n[1], n[2]);
                if (s.texcoords) {
                    const float* uv = s.texcoords + (size_t)i * 6 + v * 2;
                    t.texcoords[v] = TVector3(uv[0], uv[1], 0.0f);
                } else {
                    t.texcoords[v] = TVector3(1e30f, 1e30f, 0.0f);
                }
            }
            t.idMaterial = s.material_ids[i];
        }
        materials.resize(s.num_materials);
        for (uint32_t m = 0; m < s.num_materials; m++) {
            materials[m].color = TVector3(s.materials[m].color[0], s.materials[m].color[1], s.materials[m].color[2]);
            materials[m].eta = s.materials[m].eta;
            materials[m].brdf = s.materials[m].brdf;
        }
        lightsCDF.assign(s.light_cdf, s.light_cdf + s.num_lights);
        lightsIndices.assign(s.light_triangles, s.light_triangles + s.num_lights);
        lightsArea = s.light_area;
        bbox.min = TVector3(s.bbox_min[0], s.bbox_min[1], s.bbox_min[2]);
        bbox.max = TVector3(s.bbox_max[0], s.bbox_max[1], s.bbox_max[2]);
        return true;
    }

    void Release() {
        if (handle) sppm_mesh_destroy(handle);
        handle = nullptr;
        triangles.clear();
        materials.clear();
        lightsCDF.clear();
        lightsIndices.clear();
    }
};

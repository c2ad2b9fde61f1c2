// sppm_gpurt.hpp -- drop-in replacement of the reference's gpurt.h (class CGPURT, gpurt.h:29-67)
// for builds that keep the reference's host code (mesh.h/mesh.cpp, bvh.h/bvh.cpp, camera.h/
// camera.cpp).  Include it instead of gpurt.h, link libsppm.so, and drive frames with
// display() instead of the GLUT/OpenGL m_display().
//
// The public members the reference's main() uses keep their names and meaning: `mesh`, `camera`,
// PrecalculateMeshData() (builds the TBVH with the reference's own bvh.cpp, then uploads the
// triangles, materials, light table and the six threaded orderings through sppm_upload_scene),
// and Release().  The GL texture handles and strides are replaced by one sppm_ctx; the frame
// driver m_display() becomes display(), which queues one SPPM frame (eye pass every 10th frame,
// photon pass, hashed grid, progressive update) on the GPU.  Errors are reported through
// `status` / sppm_last_error() instead of being ignored.
#pragma once

#include <cmath>
#include <vector>

#include "bvh.h"     // the reference's TBVH
#include "camera.h"  // the reference's TCamera
#include "mesh.h"    // the reference's TMesh
#include "sppm.h"
#include "sppm_texture.h"

class CGPURT {
public:
    TMesh mesh;
    TCamera camera;
    sppm_config config;
    sppm_ctx* ctx = nullptr;
    int status = SPPM_OK;
    int device = 0;

    explicit CGPURT(unsigned resolution = 512) { sppm_config_defaults(&config, resolution); }
    ~CGPURT() { Release(); }

    // CGPURT::PrecalculateMeshData (gpurt.cpp:8-16): BVH build + upload
    int PrecalculateMeshData() {
        sppm_scene s;
        FlattenScene(&s);
        if (!ctx && (status = sppm_create(&config, device, &ctx)) != SPPM_OK) return status;
        if ((status = sppm_upload_scene(ctx, &s)) != SPPM_OK) return status;
        sppm_camera c = {};
        c.origin[0] = camera.origin.x;
        c.origin[1] = camera.origin.y;
        c.origin[2] = camera.origin.z;
        c.u[0] = camera.u.x;
        c.u[1] = camera.u.y;
        c.u[2] = camera.u.z;
        c.v[0] = camera.v.x;
        c.v[1] = camera.v.y;
        c.v[2] = camera.v.z;
        c.w[0] = camera.w.x;
        c.w[1] = camera.w.y;
        c.w[2] = camera.w.z;
        c.distance = camera.distance;
        c.width = (unsigned)camera.width;
        c.height = (unsigned)camera.height;
        return status = sppm_set_camera(ctx, &c);
    }

    // TBVH::Build with the reference's bvh.cpp, then the flat arrays of sppm_scene (valid until
    // the next call or Release)
    void FlattenScene(sppm_scene* out) {
        bvh.Build(mesh);
        const unsigned n = (unsigned)mesh.triangles.size();
        pos.resize((size_t)n * 9);
        nrm.resize((size_t)n * 9);
        tex.resize((size_t)n * 6);
        mat.resize(n);
        for (unsigned i = 0; i < n; i++) {
            const TTriangle& t = mesh.triangles[i];
            for (int v = 0; v < 3; v++) {
                pos[i * 9 + v * 3 + 0] = t.positions[v].x;
                pos[i * 9 + v * 3 + 1] = t.positions[v].y;
                pos[i * 9 + v * 3 + 2] = t.positions[v].z;
                nrm[i * 9 + v * 3 + 0] = t.normals[v].x;
                nrm[i * 9 + v * 3 + 1] = t.normals[v].y;
                nrm[i * 9 + v * 3 + 2] = t.normals[v].z;
                tex[i * 6 + v * 2 + 0] = t.texcoords[v].x;
                tex[i * 6 + v * 2 + 1] = t.texcoords[v].y;
            }
            mat[i] = t.idMaterial;
        }
        mats.resize(mesh.materials.size());
        for (size_t m = 0; m < mesh.materials.size(); m++) {
            const TMaterial& tm = mesh.materials[m];
            mats[m].color[0] = tm.color.x;
            mats[m].color[1] = tm.color.y;
            mats[m].color[2] = tm.color.z;
            mats[m].eta = tm.eta;
            mats[m].brdf = tm.brdf;
            mats[m].glossiness = 1.0f / (std::pow(2.0f / (1.0f - tm.specularity), 2.71828f) + 1.0f);  // gpurt.cpp:126
        }
        // map_Kd textures resampled to the 512x512 layers of VolumeTextureTextures (gpurt.cpp:158-198)
        mtex.assign(mesh.materials.size(), -1);
        layers.clear();
        unsigned nlayers = 0;
        const size_t layer_bytes = (size_t)SPPM_TEXTURE_RES * SPPM_TEXTURE_RES * 4;
        for (size_t m = 0; m < mesh.materials.size(); m++) {
            const TMaterial& tm = mesh.materials[m];
            if (!tm.isTextured || tm.texture.size() < (size_t)tm.textureWidth * tm.textureHeight * 3) continue;
            mtex[m] = (int32_t)nlayers++;
            layers.resize(nlayers * layer_bytes);
            sppm_tex_resample(tm.texture.data(), tm.textureWidth, tm.textureHeight,
                              layers.data() + (nlayers - 1) * layer_bytes);
        }
        const int nn = bvh.nodesNum;
        bounds.resize((size_t)nn * 6);
        tri.resize(nn);
        base.resize((size_t)6 * nn);
        miss.resize((size_t)6 * nn);
        for (int i = 0; i < nn; i++) {
            const TBBox& b = bvh.nodes[0][i].bbox;
            const float r[6] = {b.min.x, b.min.y, b.min.z, b.max.x, b.max.y, b.max.z};
            for (int k = 0; k < 6; k++) bounds[(size_t)i * 6 + k] = r[k];
            tri[i] = bvh.nodes[0][i].isLeaf ? bvh.nodes[0][i].idTriangle : -1;
        }
        for (int o = 0; o < 6; o++)
            for (int i = 0; i < nn; i++) {
                base[(size_t)o * nn + i] = bvh.nodes[o][i].idBase;
                miss[(size_t)o * nn + i] = bvh.nodes[o][i].idMiss;
            }
        sppm_scene s = {};
        s.num_triangles = n;
        s.positions = pos.data();
        s.normals = nrm.data();
        s.texcoords = tex.data();
        s.material_ids = mat.data();
        s.num_materials = (unsigned)mats.size();
        s.materials = mats.data();
        s.num_lights = (unsigned)mesh.lightsCDF.size();
        s.light_triangles = mesh.lightsIndices.data();
        s.light_cdf = mesh.lightsCDF.data();
        s.light_area = mesh.lightsCDF.empty() ? 0.0f : mesh.lightsArea;
        s.bbox_min[0] = mesh.bbox.min.x;
        s.bbox_min[1] = mesh.bbox.min.y;
        s.bbox_min[2] = mesh.bbox.min.z;
        s.bbox_max[0] = mesh.bbox.max.x;
        s.bbox_max[1] = mesh.bbox.max.y;
        s.bbox_max[2] = mesh.bbox.max.z;
        s.num_nodes = (unsigned)nn;
        s.node_bounds = bounds.data();
        s.node_triangle = tri.data();
        s.order_base = base.data();
        s.order_miss = miss.data();
        s.num_textures = nlayers;
        s.textures = nlayers ? layers.data() : nullptr;
        s.material_texture = mtex.data();
        *out = s;
    }

    // one frame of m_display (glslppm.cpp:214-536)
    int display() { return status = sppm_run_passes(ctx, 1); }

    // re.fs into a host RGB buffer (width*height*3 floats, bottom row first)
    int read_image(float* rgb, unsigned kind = SPPM_IMAGE_DISPLAY) {
        return status = sppm_read_image(ctx, kind, rgb, (size_t)config.width * config.height * 3);
    }

    // CGPURT::Release (gpurt.cpp:563-574)
    void Release() {
        if (ctx) sppm_destroy(ctx);
        ctx = nullptr;
        mesh.Release();
    }

private:
    TBVH bvh;
    std::vector<float> pos, nrm, tex, bounds;
    std::vector<int> mat, tri, base, miss;
    std::vector<sppm_material> mats;
    std::vector<uint8_t> layers;  // [textures][512][512][4]
    std::vector<int32_t> mtex;    // texture of each material or -1
};

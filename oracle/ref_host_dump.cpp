// TEST INFRASTRUCTURE (oracle side) -- never linked into the product.
//
// Runs the reference's own host code -- TMesh::LoadOBJ (mesh.cpp), TBVH::Build (bvh.cpp) and
// TCamera::Set (camera.cpp), compiled unmodified from the reference sources by oracle/build.py
// into oracle/_ref/ref_host_dump -- and writes what CGPURT::CreateTextures would pack
// (gpurt.cpp:47-552) to a flat binary file, so tests can compare the product's own loader and BVH
// builder with the reference word for word.
//
// usage: ref_host_dump <obj file name in the current directory> <scale> <out.bin>
//                      [cam_origin_xyz lookat_xyz width height fov]
// Output layout (little-endian): "SPPMREF1", then u32 counts
//   [num_triangles, num_materials, num_lights, num_nodes]
// then positions f32[n*9], normals f32[n*9], texcoords f32[n*6], material_ids i32[n],
// materials {f32 r,g,b,eta; i32 brdf; f32 glossiness}[m], light_triangles i32[l], light_cdf f32[l],
// light_area f32, bbox f32[6], node_bounds f32[nodes*6], node_triangle i32[nodes],
// order_base i32[6*nodes], order_miss i32[6*nodes], camera {f32 origin[3],u[3],v[3],w[3],distance;
// u32 width,height} (zeros when no camera arguments are given), then per material {u32 textured,
// width, height; u8 rgb[width*height*3] when textured} as LoadPPM read it.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bvh.h"
#include "camera.h"
#include "mesh.h"

static void put(FILE* f, const void* p, size_t n) {
    if (n && fwrite(p, 1, n, f) != n) {
        fprintf(stderr, "write failed\n");
        exit(2);
    }
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s file.obj scale out.bin [ox oy oz lx ly lz w h fov]\n", argv[0]);
        return 1;
    }
    const float scale = (float)atof(argv[2]);
    TMesh mesh;
    mesh.lightsArea = 0.0f;  // static storage in the reference (CGPURT gpurt is a global)
    mesh.LoadOBJ(argv[1], TVector3(0.0f, 0.0f, 0.0f), scale);
    TBVH bvh;
    bvh.Build(mesh);

    FILE* f = fopen(argv[3], "wb");
    if (!f) return 2;
    put(f, "SPPMREF1", 8);
    const unsigned n = (unsigned)mesh.triangles.size();
    const unsigned counts[4] = {n, (unsigned)mesh.materials.size(), (unsigned)mesh.lightsCDF.size(),
                                (unsigned)bvh.nodesNum};
    put(f, counts, sizeof(counts));
    std::vector<float> pos, nrm, tex;
    std::vector<int> mat;
    for (unsigned i = 0; i < n; i++) {
        const TTriangle& t = mesh.triangles[i];
        for (int v = 0; v < 3; v++) {
            pos.push_back(t.positions[v].x);
            pos.push_back(t.positions[v].y);
            pos.push_back(t.positions[v].z);
            nrm.push_back(t.normals[v].x);
            nrm.push_back(t.normals[v].y);
            nrm.push_back(t.normals[v].z);
            tex.push_back(t.texcoords[v].x);
            tex.push_back(t.texcoords[v].y);
        }
        mat.push_back(t.idMaterial);
    }
    put(f, pos.data(), pos.size() * 4);
    put(f, nrm.data(), nrm.size() * 4);
    put(f, tex.data(), tex.size() * 4);
    put(f, mat.data(), mat.size() * 4);
    for (size_t i = 0; i < mesh.materials.size(); i++) {
        const TMaterial& m = mesh.materials[i];
        // the packed glossiness of gpurt.cpp:126 (the GL packer itself cannot be compiled here);
        // meaningless for the default material, whose specularity the reference never sets
        const float g = 1.0f / (pow(2.0f / (1.0f - m.specularity), 2.71828f) + 1.0f);
        const float rec[4] = {m.color.x, m.color.y, m.color.z, m.eta};
        put(f, rec, 16);
        put(f, &m.brdf, 4);
        put(f, &g, 4);
    }
    put(f, mesh.lightsIndices.data(), mesh.lightsIndices.size() * 4);
    put(f, mesh.lightsCDF.data(), mesh.lightsCDF.size() * 4);
    put(f, &mesh.lightsArea, 4);
    const float bb[6] = {mesh.bbox.min.x, mesh.bbox.min.y, mesh.bbox.min.z,
                         mesh.bbox.max.x, mesh.bbox.max.y, mesh.bbox.max.z};
    put(f, bb, sizeof(bb));
    const int nn = bvh.nodesNum;
    for (int i = 0; i < nn; i++) {
        const TBBox& b = bvh.nodes[0][i].bbox;
        const float r[6] = {b.min.x, b.min.y, b.min.z, b.max.x, b.max.y, b.max.z};
        put(f, r, sizeof(r));
    }
    for (int i = 0; i < nn; i++) {
        const int tri = bvh.nodes[0][i].isLeaf ? bvh.nodes[0][i].idTriangle : -1;
        put(f, &tri, 4);
    }
    for (int o = 0; o < 6; o++)
        for (int i = 0; i < nn; i++) put(f, &bvh.nodes[o][i].idBase, 4);
    for (int o = 0; o < 6; o++)
        for (int i = 0; i < nn; i++) put(f, &bvh.nodes[o][i].idMiss, 4);

    float camrec[13] = {0};
    unsigned camwh[2] = {0, 0};
    if (argc >= 13) {
        TCamera cam;
        const TVector3 o((float)atof(argv[4]), (float)atof(argv[5]), (float)atof(argv[6]));
        const TVector3 l((float)atof(argv[7]), (float)atof(argv[8]), (float)atof(argv[9]));
        cam.Set(o, l, atoi(argv[10]), atoi(argv[11]), (float)atof(argv[12]));
        const float r[13] = {cam.origin.x, cam.origin.y, cam.origin.z, cam.u.x, cam.u.y, cam.u.z,
                             cam.v.x, cam.v.y, cam.v.z, cam.w.x, cam.w.y, cam.w.z, cam.distance};
        memcpy(camrec, r, sizeof(r));
        camwh[0] = (unsigned)cam.width;
        camwh[1] = (unsigned)cam.height;
    }
    put(f, camrec, sizeof(camrec));
    put(f, camwh, sizeof(camwh));
    // material textures as LoadPPM read them: per material u32 textured, width, height, RGB8 bytes
    for (size_t i = 0; i < mesh.materials.size(); i++) {
        const TMaterial& m = mesh.materials[i];
        const unsigned rec[3] = {m.isTextured ? 1u : 0u, (unsigned)m.textureWidth, (unsigned)m.textureHeight};
        put(f, rec, sizeof(rec));
        if (m.isTextured) put(f, m.texture.data(), m.texture.size());
    }
    fclose(f);
    return 0;
}

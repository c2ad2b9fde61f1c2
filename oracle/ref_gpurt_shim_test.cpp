// TEST INFRASTRUCTURE: compiles include/sppm_gpurt.hpp (the drop-in for gpurt.h) together with the
// reference's own mesh.cpp / bvh.cpp / camera.cpp and libsppm.so, loads an OBJ the way the
// reference's main() does (glslppm.cpp:801-819), flattens it and writes the sppm_scene arrays in
// the ref_host_dump format; with a GPU it also renders frames through the C ABI.
// usage: ref_gpurt_shim_test <obj in cwd> <scale> <out.bin> <frames>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sppm_gpurt.hpp"

static void put(FILE* f, const void* p, size_t n) {
    if (n) fwrite(p, 1, n, f);
}

int main(int argc, char** argv) {
    if (argc < 5) return 1;
    CGPURT gpurt(16);
    gpurt.mesh.lightsArea = 0.0f;
    gpurt.mesh.LoadOBJ(argv[1], TVector3(0.0f, 0.0f, 0.0f), (float)atof(argv[2]));
    gpurt.camera.Set(TVector3(0.0f, 0.0f, 13.0f), TVector3(0.0f, 0.0f, 0.0f), 16, 16, 45.0f);
    sppm_scene s;
    gpurt.FlattenScene(&s);
    FILE* f = fopen(argv[3], "wb");
    if (!f) return 2;
    put(f, "SPPMREF1", 8);
    const unsigned counts[4] = {s.num_triangles, s.num_materials, s.num_lights, s.num_nodes};
    put(f, counts, 16);
    put(f, s.positions, (size_t)s.num_triangles * 36);
    put(f, s.normals, (size_t)s.num_triangles * 36);
    put(f, s.texcoords, (size_t)s.num_triangles * 24);
    put(f, s.material_ids, (size_t)s.num_triangles * 4);
    put(f, s.materials, (size_t)s.num_materials * sizeof(sppm_material));
    put(f, s.light_triangles, (size_t)s.num_lights * 4);
    put(f, s.light_cdf, (size_t)s.num_lights * 4);
    put(f, &s.light_area, 4);
    put(f, s.bbox_min, 12);
    put(f, s.bbox_max, 12);
    put(f, s.node_bounds, (size_t)s.num_nodes * 24);
    put(f, s.node_triangle, (size_t)s.num_nodes * 4);
    put(f, s.order_base, (size_t)s.num_nodes * 24);
    put(f, s.order_miss, (size_t)s.num_nodes * 24);
    const float cam[13] = {0};
    const unsigned wh[2] = {0, 0};
    put(f, cam, sizeof(cam));
    put(f, wh, sizeof(wh));
    // per material: the flattened texture layer as a 512x512 RGB8 record (textured flag, 512, 512)
    for (unsigned m = 0; m < s.num_materials; m++) {
        const int layer = s.material_texture ? s.material_texture[m] : -1;
        const unsigned rec[3] = {layer >= 0 ? 1u : 0u, 512u, 512u};
        put(f, rec, sizeof(rec));
        if (layer < 0) continue;
        std::vector<unsigned char> rgb((size_t)512 * 512 * 3);
        const unsigned char* src = s.textures + (size_t)layer * 512 * 512 * 4;
        for (size_t i = 0; i < (size_t)512 * 512; i++)
            for (int c = 0; c < 3; c++) rgb[i * 3 + c] = src[i * 4 + c];
        put(f, rgb.data(), rgb.size());
    }
    fclose(f);
    const int frames = atoi(argv[4]);
    if (frames > 0) {
        if (gpurt.PrecalculateMeshData() != SPPM_OK) {
            char msg[512];
            sppm_last_error(msg, sizeof msg);
            printf("status %d: %s\n", gpurt.status, msg);
            return gpurt.status;
        }
        for (int i = 0; i < frames; i++) gpurt.display();
        std::vector<float> rgb(16 * 16 * 3);
        if (gpurt.read_image(rgb.data()) != SPPM_OK) return 3;
        printf("rendered %d frames\n", frames);
    }
    return 0;
}

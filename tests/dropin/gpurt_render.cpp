// TEST INFRASTRUCTURE: renders through the drop-in CGPURT of include/sppm_gpurt.hpp the way the
// reference's main() and m_display() drive CGPURT (glslppm.cpp:801-835, 214-536): load an OBJ into
// gpurt.mesh, set gpurt.camera, PrecalculateMeshData(), display() once per frame, then read the
// linear radiance image into a file (width*height*3 floats).
// usage: gpurt_render <obj> <scale> <resolution> <frames> <radius_fraction> <ox oy oz lx ly lz fov>
//        <out.bin>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sppm_gpurt.hpp"

int main(int argc, char** argv) {
    if (argc < 14) {
        fprintf(stderr, "usage: %s obj scale res frames radius_fraction ox oy oz lx ly lz fov out.bin\n", argv[0]);
        return 1;
    }
    const unsigned res = (unsigned)atoi(argv[3]);
    const int frames = atoi(argv[4]);
    CGPURT gpurt(res);
    gpurt.config.radius_rule = SPPM_RADIUS_DIAGONAL;
    gpurt.config.radius_fraction = (float)atof(argv[5]);
    if (!gpurt.mesh.LoadOBJ(argv[1], TVector3(0.0f, 0.0f, 0.0f), (float)atof(argv[2]))) return 2;
    gpurt.camera.Set(TVector3((float)atof(argv[6]), (float)atof(argv[7]), (float)atof(argv[8])),
                     TVector3((float)atof(argv[9]), (float)atof(argv[10]), (float)atof(argv[11])), (int)res, (int)res,
                     (float)atof(argv[12]));
    if (gpurt.PrecalculateMeshData() != SPPM_OK) {
        char msg[512];
        sppm_last_error(msg, sizeof msg);
        fprintf(stderr, "status %d: %s\n", gpurt.status, msg);
        return 3;
    }
    for (int i = 0; i < frames; i++)
        if (gpurt.display() != SPPM_OK) return 4;
    std::vector<float> rgb((size_t)res * res * 3);
    if (gpurt.read_image(rgb.data(), SPPM_IMAGE_RADIANCE) != SPPM_OK) return 5;
    FILE* f = fopen(argv[13], "wb");
    if (!f) return 6;
    fwrite(rgb.data(), 4, rgb.size(), f);
    fclose(f);
    printf("rendered %d frames through CGPURT\n", frames);
    return 0;
}

// TEST INFRASTRUCTURE: a stand-in for the reference's bvh.h (TBVH with six threaded orderings) with
// the members include/sppm_gpurt.hpp reads, filled by this library's exact-SAH builder
// (sppm_mesh_build_bvh, node for node the reference's tree).
#pragma once

#include <vector>

#include "mesh.h"

struct TBVHNode {
    TBBox bbox;
    bool isLeaf = false;
    int idTriangle = -1, idBase = 0, idMiss = -1;
};

class TBVH {
public:
    std::vector<TBVHNode> storage[6];
    TBVHNode* nodes[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int nodesNum = 0;

    void Build(TMesh& mesh) {
        nodesNum = 0;
        if (!mesh.handle || sppm_mesh_build_bvh(mesh.handle) != SPPM_OK) return;
        sppm_scene s;
        if (sppm_mesh_get_scene(mesh.handle, &s) != SPPM_OK) return;
        const int nn = (int)s.num_nodes;
        for (int o = 0; o < 6; o++) {
            storage[o].assign(nn, TBVHNode{});
            nodes[o] = storage[o].data();
            for (int i = 0; i < nn; i++) {
                TBVHNode& d = storage[o][i];
                // ordering o's i-th node is the canonical node idBase; bounds and leaves live on
                // the canonical node (ordering 0 is the canonical numbering)
                d.idBase = s.order_base[(size_t)o * nn + i];
                d.idMiss = s.order_miss[(size_t)o * nn + i];
                const int c = o == 0 ? i : d.idBase;
                const float* b = s.node_bounds + (size_t)c * 6;
                d.bbox.min = TVector3(b[0], b[1], b[2]);
                d.bbox.max = TVector3(b[3], b[4], b[5]);
                d.idTriangle = s.node_triangle[c];
                d.isLeaf = d.idTriangle >= 0;
            }
        }
        nodesNum = nn;
    }
};

// Host BVH construction with the semantics of TBVH::Build (bvh.cpp:244-317), and the look-at
// camera of TCamera::Set (camera.cpp:4-18).
//
// The shader path traverses six "threaded" orderings of one binary BVH (one per major ray
// direction).  The tree, its node numbering and its miss links determine the order in which
// triangles are tested and therefore which of two triangles at exactly the same distance is
// reported, so this builder reproduces the reference's tree node for node:
//  * exact-SAH split: for each axis in turn the index range is quicksorted by centroid with a
//    middle-element pivot and Hoare partitioning (bvh.cpp:7-29) -- the ranges are sorted in
//    place one after the other, so ties keep the order the previous axis left; a left sweep and a
//    right sweep of box areas give cost = nL*areaL + nR*areaR, and the first strictly smaller cost
//    wins (bvh.cpp:81-150); two triangles split trivially (:67-78); one triangle per leaf (:39-57);
//  * children are ordered so that the one with the smaller min.x comes first (:159-168) and the
//    nodes are numbered in preorder;
//  * orderings 1..5 (-x, +y, -y, +z, -z) swap the children of every internal node unless
//    left.max.x > right.max.x, left.min.y < right.min.y, left.max.y > right.max.y,
//    left.min.z < right.min.z, left.max.z > right.max.z respectively (:287-301), and renumber in
//    preorder (:178-208);
//  * miss links: a leaf's is the next node in preorder, a left child's is its sibling, a right
//    child's is its parent's, the root's is -1 (:211-241, 310-315).
// Recursion is replaced by explicit stacks (the result does not depend on the order in which
// disjoint ranges are processed), so deep trees of multi-million-triangle meshes do not overflow
// the host stack.
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "scene_internal.h"

using sppm::Box;
using sppm::V3;
using sppm::v3;

namespace {

float comp(V3 v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }

// in-place quicksort of idx[li..ri] by centroid component `axis`
void sort_axis(const std::vector<V3>& cent, int* idx, int axis, int li, int ri, std::vector<std::pair<int, int>>& stack) {
    stack.clear();
    stack.push_back({li, ri});
    while (!stack.empty()) {
        const int l = stack.back().first, r = stack.back().second;
        stack.pop_back();
        int i = l, j = r;
        const float pivot = comp(cent[idx[(l + r) / 2]], axis);
        for (;;) {
            while (comp(cent[idx[i]], axis) < pivot) i++;
            while (comp(cent[idx[j]], axis) > pivot) j--;
            if (i >= j) break;
            std::swap(idx[i], idx[j]);
            i++;
            j--;
        }
        if (l < i - 1) stack.push_back({l, i - 1});
        if (j + 1 < r) stack.push_back({j + 1, r});
    }
}

struct Node {
    Box box;
    bool leaf = false;
    int left = -1, right = -1, tri = -1;
};

struct Task {
    int lo, n;
    Box box;
    int parent, side;  // side 0 = left child, 1 = right child
};

// preorder numbering + miss links of one ordering; `nodes` hold children in that ordering
void thread_ordering(const std::vector<Node>& nodes, int32_t* base, int32_t* miss) {
    const int n = (int)nodes.size();
    std::vector<int> pos_of(n, -1);
    // preorder walk: base[p] = canonical id
    std::vector<int> stack;
    stack.push_back(0);
    int p = 0;
    while (!stack.empty()) {
        const int c = stack.back();
        stack.pop_back();
        base[p] = c;
        pos_of[c] = p;
        p++;
        if (!nodes[c].leaf) {
            stack.push_back(nodes[c].right);
            stack.push_back(nodes[c].left);
        }
    }
    // miss links in preorder (parents before children)
    for (int i = 0; i < n; i++) miss[i] = -1;
    for (int q = 0; q < n; q++) {
        const Node& nd = nodes[base[q]];
        if (nd.leaf) {
            miss[q] = q + 1;
            continue;
        }
        const int lp = pos_of[nd.left], rp = pos_of[nd.right];
        // left child -> sibling; right child -> parent's miss (root's miss stays -1)
        if (!nodes[nd.left].leaf) miss[lp] = rp;
        if (!nodes[nd.right].leaf) miss[rp] = miss[q];
    }
}

}  // namespace

extern "C" int sppm_mesh_build_bvh(sppm_mesh* m) {
    if (!m) return sppm::fail(SPPM_ERR_ARG, "sppm_mesh_build_bvh: null mesh");
    const int nt = (int)m->num_triangles;
    if (nt < 1) return sppm::fail(SPPM_ERR_ARG, "sppm_mesh_build_bvh: mesh has no triangles");
    const int nn = 2 * nt - 1;
    std::vector<Node> nodes(nn);
    std::vector<int> idx(nt), sorted(nt);
    for (int i = 0; i < nt; i++) idx[i] = i;
    std::vector<float> left_area(nt);
    std::vector<Box> lbox(nt);
    std::vector<std::pair<int, int>> qstack;
    std::vector<Task> tasks;
    tasks.push_back({0, nt, m->bbox, -1, 0});
    int counter = 0;
    while (!tasks.empty()) {
        const Task t = tasks.back();
        tasks.pop_back();
        if (counter >= nn) return sppm::fail(SPPM_ERR_STATE, "sppm_mesh_build_bvh: node overflow");
        const int id = counter++;
        if (t.parent >= 0) (t.side == 0 ? nodes[t.parent].left : nodes[t.parent].right) = id;
        nodes[id].box = t.box;
        if (t.n <= 1) {
            nodes[id].leaf = true;
            nodes[id].tri = t.n ? idx[t.lo] : -1;
            continue;
        }
        int best_index = 0;
        Box best_l, best_r;
        best_l.init();
        best_r.init();
        int* seg = &idx[t.lo];
        if (t.n == 2) {
            best_l = m->tri_bbox[seg[0]];
            best_r = m->tri_bbox[seg[1]];
        } else {
            float best_cost = 1e+30f;
            int best_axis = 0;
            for (int k = 0; k <= 2; k++) {
                sort_axis(m->tri_centroid, seg, k, 0, t.n - 1, qstack);
                Box bl, br;
                bl.init();
                for (int i = 0; i < t.n; i++) {
                    const Box& tb = m->tri_bbox[seg[i]];
                    bl.expand(tb.mn);
                    bl.expand(tb.mx);
                    left_area[i] = bl.area();
                    lbox[i] = bl;
                }
                int tri_num = t.n - 1;
                br.init();
                for (int j = t.n - 2; j >= 0; j--) {
                    const Box& tb = m->tri_bbox[seg[j + 1]];
                    br.expand(tb.mn);
                    br.expand(tb.mx);
                    const float cost = (float)tri_num * left_area[j] + (float)(t.n - tri_num) * br.area();
                    if (cost < best_cost) {
                        best_cost = cost;
                        best_axis = k;
                        best_index = j;
                        best_l = lbox[j];
                        best_r = br;
                    }
                    tri_num--;
                }
                if (best_axis == k) memcpy(sorted.data(), seg, sizeof(int) * t.n);
            }
            memcpy(seg, sorted.data(), sizeof(int) * t.n);
        }
        const Task tl{t.lo, best_index + 1, best_l, id, 0};
        const Task tr{t.lo + best_index + 1, t.n - (best_index + 1), best_r, id, 1};
        // canonical child order: smaller min.x first; push the second child first (stack)
        if (best_l.mn.x < best_r.mn.x) {
            tasks.push_back({tr.lo, tr.n, tr.box, id, 1});
            tasks.push_back({tl.lo, tl.n, tl.box, id, 0});
        } else {
            tasks.push_back({tl.lo, tl.n, tl.box, id, 1});
            tasks.push_back({tr.lo, tr.n, tr.box, id, 0});
        }
    }
    if (counter != nn) return sppm::fail(SPPM_ERR_STATE, "sppm_mesh_build_bvh: %d nodes, expected %d", counter, nn);

    m->num_nodes = (uint32_t)nn;
    m->node_bounds.resize((size_t)nn * 6);
    m->node_triangle.resize(nn);
    for (int i = 0; i < nn; i++) {
        const Box& b = nodes[i].box;
        float* o = &m->node_bounds[(size_t)i * 6];
        o[0] = b.mn.x;
        o[1] = b.mn.y;
        o[2] = b.mn.z;
        o[3] = b.mx.x;
        o[4] = b.mx.y;
        o[5] = b.mx.z;
        m->node_triangle[i] = nodes[i].leaf ? nodes[i].tri : -1;
    }
    m->order_base.resize((size_t)6 * nn);
    m->order_miss.resize((size_t)6 * nn);
    for (int face = 0; face < 6; face++) {
        std::vector<Node> ord = nodes;  // children in the order of this face
        if (face != 0) {
            for (int i = 0; i < nn; i++) {
                Node& nd = ord[i];
                if (nd.leaf) continue;
                const Box& l = nodes[nd.left].box;
                const Box& r = nodes[nd.right].box;
                bool keep;
                switch (face) {
                    case 1: keep = l.mx.x > r.mx.x; break;
                    case 2: keep = l.mn.y < r.mn.y; break;
                    case 3: keep = l.mx.y > r.mx.y; break;
                    case 4: keep = l.mn.z < r.mn.z; break;
                    default: keep = l.mx.z > r.mx.z; break;
                }
                if (!keep) std::swap(nd.left, nd.right);
            }
        }
        thread_ordering(ord, &m->order_base[(size_t)face * nn], &m->order_miss[(size_t)face * nn]);
    }
    return SPPM_OK;
}

extern "C" void sppm_camera_look_at(sppm_camera* cam, const float origin[3], const float lookat[3],
                                    uint32_t width, uint32_t height, float fov_degrees) {
    if (!cam || !origin || !lookat) return;
    cam->origin[0] = origin[0];
    cam->origin[1] = origin[1];
    cam->origin[2] = origin[2];
    cam->width = width;
    cam->height = height;
    cam->distance = float(height) / (2.0f * tanf((fov_degrees / 2.0f) * (3.141592f / 180.0f)));
    const V3 tv = v3(0.0f, 1.0f, 0.0f);
    const V3 w = sppm::normalize3(v3(lookat[0], lookat[1], lookat[2]) - v3(origin[0], origin[1], origin[2]));
    const V3 u = sppm::normalize3(sppm::cross3(tv, w));
    const V3 v = sppm::normalize3(sppm::cross3(w, u));
    cam->u[0] = u.x;
    cam->u[1] = u.y;
    cam->u[2] = u.z;
    cam->v[0] = v.x;
    cam->v[1] = v.y;
    cam->v[2] = v.z;
    cam->w[0] = w.x;
    cam->w[1] = w.y;
    cam->w[2] = w.z;
}

// 4-wide BVH with 8-bit quantised child boxes for the mixed-precision path.
//
// Built from the binary SAH BVH of sppm_mesh_build_bvh (the reference's tree): each 4-wide node
// takes a binary node's two children and repeatedly opens its internal child of largest surface
// area until it holds four children or only leaves.  Child boxes are stored relative to the node's
// box as 8-bit integers per bound and axis, with a power-of-two scale per axis (the layout of
// compressed wide BVHs, Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs
// Through Compressed Wide BVHs", HPG 2017).  Bounds are rounded outward, and every decoded bound
// -- computed exactly as the kernel does, fma(q, 2^e, origin) -- is checked to enclose the
// child's float box, so a traversal over the quantised boxes never misses a triangle the exact
// boxes would reach.
#include <cmath>
#include <cstring>
#include <vector>

#include "scene_internal.h"
#include "scene_bvh4.h"

namespace sppm {

namespace {

struct BNode {
    Box box;
    int left = -1, right = -1, tri = -1;  // leaf: tri >= 0
};

float area(const Box& b) { return b.area(); }

// smallest power-of-two exponent e with extent / 2^e <= 255
int scale_exponent(float extent) {
    if (!(extent > 0.0f)) return -126;
    int e = (int)std::ceil(std::log2((double)extent / 255.0));
    if (e < -126) e = -126;
    while (std::ldexp(255.0, e) < (double)extent) e++;
    return e;
}

}  // namespace

int build_bvh4(const sppm_scene& s, std::vector<Node4>& out, uint32_t* max_depth) {
    const int nn = (int)s.num_nodes;
    if (nn < 1) return -1;
    // binary tree from ordering 0 (canonical preorder): left = i + 1, right = miss link of left
    std::vector<BNode> b(nn);
    for (int i = 0; i < nn; i++) {
        const float* bb = s.node_bounds + (size_t)i * 6;
        b[i].box.mn = v3(bb[0], bb[1], bb[2]);
        b[i].box.mx = v3(bb[3], bb[4], bb[5]);
        b[i].tri = s.node_triangle[i];
    }
    const int32_t* base0 = s.order_base;
    const int32_t* miss0 = s.order_miss;
    for (int i = 0; i < nn; i++) {
        if (base0[i] != i) return -2;  // ordering 0 is the canonical numbering
        if (b[i].tri >= 0) continue;
        if (i + 1 >= nn) return -3;
        b[i].left = i + 1;
        b[i].right = miss0[i + 1];
        if (b[i].right <= i + 1 || b[i].right >= nn) return -4;
    }
    out.clear();
    uint32_t depth_max = 0;
    // breadth-first: a 4-wide node per binary internal node reached as a collapsed child
    struct Item {
        int bnode;
        int slot;  // index in out
        uint32_t depth;
    };
    std::vector<Item> queue;
    out.push_back(Node4{});
    queue.push_back({0, 0, 1});  // a single-triangle scene: the root holds one leaf child
    for (size_t qi = 0; qi < queue.size(); qi++) {
        const Item it = queue[qi];
        depth_max = it.depth > depth_max ? it.depth : depth_max;
        std::vector<int> kids;
        if (b[it.bnode].tri >= 0) {
            kids.push_back(it.bnode);
        } else {
            kids.push_back(b[it.bnode].left);
            kids.push_back(b[it.bnode].right);
            while (kids.size() < 4) {
                int best = -1;
                float best_area = -1.0f;
                for (size_t k = 0; k < kids.size(); k++) {
                    if (b[kids[k]].tri >= 0) continue;
                    const float a = area(b[kids[k]].box);
                    if (a > best_area) {
                        best_area = a;
                        best = (int)k;
                    }
                }
                if (best < 0) break;
                const int open = kids[best];
                kids[best] = b[open].left;
                kids.insert(kids.begin() + best + 1, b[open].right);
            }
        }
        Node4 node;
        memset(&node, 0, sizeof(node));
        const Box& nb = b[it.bnode].box;
        node.origin[0] = nb.mn.x;
        node.origin[1] = nb.mn.y;
        node.origin[2] = nb.mn.z;
        const float ext[3] = {nb.mx.x - nb.mn.x, nb.mx.y - nb.mn.y, nb.mx.z - nb.mn.z};
        int e[3];
        for (int a = 0; a < 3; a++) {
            e[a] = scale_exponent(ext[a]);
            node.exponent[a] = (uint8_t)(e[a] + 127);
        }
        node.count = (uint8_t)kids.size();
        for (size_t k = 0; k < 4; k++) node.child[k] = kChildEmpty;
        for (size_t k = 0; k < kids.size(); k++) {
            const BNode& c = b[kids[k]];
            const float lo[3] = {c.box.mn.x, c.box.mn.y, c.box.mn.z};
            const float hi[3] = {c.box.mx.x, c.box.mx.y, c.box.mx.z};
            for (int a = 0; a < 3; a++) {
                const float sc = std::ldexp(1.0f, e[a]);
                const float o = node.origin[a];
                double ql = std::floor(((double)lo[a] - (double)o) / (double)sc);
                double qh = std::ceil(((double)hi[a] - (double)o) / (double)sc);
                ql = ql < 0 ? 0 : (ql > 255 ? 255 : ql);
                qh = qh < 0 ? 0 : (qh > 255 ? 255 : qh);
                // decoded exactly as the kernel decodes; move outward until it encloses
                while (ql > 0 && std::fma((float)ql, sc, o) > lo[a]) ql -= 1;
                while (qh < 255 && std::fma((float)qh, sc, o) < hi[a]) qh += 1;
                if (std::fma((float)ql, sc, o) > lo[a] || std::fma((float)qh, sc, o) < hi[a]) return -5;
                node.qlo[a][k] = (uint8_t)ql;
                node.qhi[a][k] = (uint8_t)qh;
            }
            if (c.tri >= 0) node.child[k] = ~c.tri;  // leaf: one triangle
        }
        // internal children get consecutive slots at the end of the queue
        for (size_t k = 0; k < kids.size(); k++) {
            if (b[kids[k]].tri >= 0) continue;
            const int slot = (int)out.size();
            out.push_back(Node4{});
            node.child[k] = slot;
            queue.push_back({kids[k], slot, it.depth + 1});
        }
        out[it.slot] = node;
    }
    if (max_depth) *max_depth = depth_max;
    return 0;
}

}  // namespace sppm

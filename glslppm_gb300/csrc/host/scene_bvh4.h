// 4-wide quantised BVH of the mixed-precision path (layout shared by the host builder and the
// kernels).
#pragma once

#include <cstdint>
#include <vector>

#include "sppm.h"

namespace sppm {

constexpr int32_t kChildEmpty = INT32_MIN;  // unused child slot
constexpr uint32_t kBvh4MaxDepth = 64;      // traversal stack holds 3 entries per level

// 64 bytes: a child k's box is origin + q * 2^(exponent - 127) per axis, q in [qlo, qhi]
struct alignas(16) Node4 {
    float origin[3];
    uint8_t exponent[3];  // biased by 127 (the float exponent field of the scale)
    uint8_t count;        // children in use
    int32_t child[4];     // >= 0: 4-wide node index; < 0: ~triangle index (a leaf); kChildEmpty
    uint8_t qlo[3][4];    // [axis][child]
    uint8_t qhi[3][4];
    uint8_t pad[8];
};
static_assert(sizeof(Node4) == 64, "Node4 is 64 bytes");

// Builds the 4-wide BVH from the binary one carried by the scene (ordering 0).  Returns 0, or a
// negative value when the scene's BVH arrays are inconsistent or a bound cannot be quantised.
int build_bvh4(const sppm_scene& s, std::vector<Node4>& out, uint32_t* max_depth);

}  // namespace sppm

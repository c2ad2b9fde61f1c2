// GPU construction of the threaded BVH arrays (sppm_mesh_build_bvh_gpu, sppm_mesh_build_bvh_gpu_ex).
//
// The host builder (csrc/host/scene_bvh.cpp) reproduces the reference's exact-SAH tree node for
// node, which costs seconds per million triangles.  These builders make a different tree in the
// same layout, in milliseconds:
//  1. 30-bit Morton code of each triangle centroid in the scene box; triangles sorted by
//     (code, index);
//  2a. PLOC (the default): parallel locally-ordered clustering (Meister and Bittner, "Parallel
//     Locally-Ordered Clustering for Bounding Volume Hierarchy Construction", IEEE TVCG 2018).
//     The sorted leaves are the first clusters; every round, each cluster finds the neighbour
//     within kPlocRadius positions of the cluster order whose union box has the smallest surface
//     area (ties to the lower position, so the closest pair overall is always mutual), mutual
//     pairs merge into a new node, and the clusters are compacted in order; the rounds end with
//     one cluster.  The tree approaches a full SAH sweep's quality;
//  2b. the radix tree over the sorted codes (Karras, "Maximizing parallelism in the construction
//     of BVHs, octrees, and k-d trees", HPG 2012), then boxes and subtree sizes bottom-up (the
//     second child to finish computes its parent): faster to build, more nodes per ray;
//  3. the six threaded orderings of the reference's layout (bvh.cpp:159-168, 287-315): canonical
//     child order = smaller min.x first, orderings 1..5 keep that order only when the face's
//     predicate holds, nodes numbered in preorder; each node finds its preorder position by
//     walking to the root (position = sum over ancestors of 1 + the node count of the sibling
//     subtree that precedes it; a subtree of k leaves has 2k-1 nodes), and its miss link is the
//     node that follows its subtree.
// Triangle sorting and cluster compaction use cub (the CUDA toolkit's device primitives).
#include <cstdint>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>
#include <cuda_runtime.h>

#include "../host/scene_internal.h"
#include "runtime.h"

using sppm::fail;

namespace {

struct GBox {
    float mn[3], mx[3];
};

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {  // 10 bits -> every third bit
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const float* __restrict__ centroid, uint32_t n, float3 lo, float3 inv_ext,
                         uint32_t* __restrict__ code, uint32_t* __restrict__ index) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = fminf(fmaxf((centroid[3 * i + 0] - lo.x) * inv_ext.x, 0.0f), 1.0f);
    const float y = fminf(fmaxf((centroid[3 * i + 1] - lo.y) * inv_ext.y, 0.0f), 1.0f);
    const float z = fminf(fmaxf((centroid[3 * i + 2] - lo.z) * inv_ext.z, 0.0f), 1.0f);
    const uint32_t xi = min((uint32_t)(x * 1024.0f), 1023u), yi = min((uint32_t)(y * 1024.0f), 1023u),
                   zi = min((uint32_t)(z * 1024.0f), 1023u);
    code[i] = (expand_bits10(xi) << 2) | (expand_bits10(yi) << 1) | expand_bits10(zi);
    index[i] = i;
}

// length of the common prefix of sorted keys i and j (position breaks ties); -1 outside [0, n)
__device__ __forceinline__ int delta(const uint32_t* code, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = code[i], b = code[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// node numbering: internal nodes 0 .. n-2, leaf k = n-1+k (k-th sorted triangle)
__global__ void k_radix_tree(const uint32_t* __restrict__ code, int n, int32_t* __restrict__ left,
                             int32_t* __restrict__ right, int32_t* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = delta(code, n, i, i + 1) - delta(code, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = delta(code, n, i, i - d);
    int lmax = 2;
    while (delta(code, n, i, i + lmax * d) > dmin) {
        lmax <<= 1;
        if (lmax > 2 * n) break;  // bounded: the range cannot exceed the key count
    }
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(code, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(code, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(code, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int L = lo == gamma ? (n - 1) + gamma : gamma;
    const int R = hi == gamma + 1 ? (n - 1) + gamma + 1 : gamma + 1;
    left[i] = L;
    right[i] = R;
    parent[L] = i;
    parent[R] = i;
    if (i == 0) parent[0] = -1;
}

__global__ void k_bounds(const uint32_t* __restrict__ sorted_tri, const GBox* __restrict__ tri_box, int n,
                         const int32_t* __restrict__ left, const int32_t* __restrict__ right,
                         const int32_t* __restrict__ parent, GBox* __restrict__ box, int32_t* __restrict__ size,
                         uint32_t* __restrict__ arrivals) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int node = (n - 1) + k;
    box[node] = tri_box[sorted_tri[k]];
    size[node] = 1;
    if (n == 1) return;
    for (int steps = 0; steps < n; steps++) {  // bounded by the tree depth (< n)
        __threadfence();
        const int p = parent[node];
        if (p < 0) break;
        if (atomicAdd(&arrivals[p], 1u) == 0) break;  // the sibling is not done yet: it continues
        __threadfence();
        // the sibling's results were written by another thread: read them past L1
        const float* a = reinterpret_cast<const float*>(box + left[p]);
        const float* b = reinterpret_cast<const float*>(box + right[p]);
        GBox u;
        for (int c = 0; c < 3; c++) {
            u.mn[c] = fminf(__ldcg(a + c), __ldcg(b + c));
            u.mx[c] = fmaxf(__ldcg(a + 3 + c), __ldcg(b + 3 + c));
        }
        box[p] = u;
        size[p] = __ldcg(size + left[p]) + __ldcg(size + right[p]);
        node = p;
    }
}

// ---- PLOC ------------------------------------------------------------------------------------
constexpr int kPlocRadius = 16;
constexpr int kPlocBlock = 256;

__device__ __forceinline__ GBox box_union(const GBox& a, const GBox& b) {
    GBox u;
    for (int c = 0; c < 3; c++) {
        u.mn[c] = fminf(a.mn[c], b.mn[c]);
        u.mx[c] = fmaxf(a.mx[c], b.mx[c]);
    }
    return u;
}

__device__ __forceinline__ float box_area(const GBox& b) {
    const float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    return dx * dy + dy * dz + dz * dx;  // half the surface area: only the order matters
}

// leaf k (sorted position) = node n-1+k; the first clusters are the leaves in Morton order
__global__ void k_ploc_leaves(const uint32_t* __restrict__ sorted_tri, const GBox* __restrict__ tri_box, int n,
                              GBox* __restrict__ box, int32_t* __restrict__ size, int32_t* __restrict__ cluster) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int node = (n - 1) + k;
    box[node] = tri_box[sorted_tri[k]];
    size[node] = 1;
    cluster[k] = node;
}

// each cluster's nearest neighbour within kPlocRadius positions (smallest union area; ties to the
// lower position); the window's boxes are staged in shared memory
__global__ void __launch_bounds__(kPlocBlock) k_ploc_nearest(const int32_t* __restrict__ cluster, int nc,
                                                           const GBox* __restrict__ box, int32_t* __restrict__ nearest) {
    __shared__ GBox sb[kPlocBlock + 2 * kPlocRadius];
    const int b0 = blockIdx.x * kPlocBlock;
    for (int t = threadIdx.x; t < kPlocBlock + 2 * kPlocRadius; t += kPlocBlock) {
        const int g = b0 - kPlocRadius + t;
        if (g >= 0 && g < nc) sb[t] = box[cluster[g]];
    }
    __syncthreads();
    const int i = b0 + (int)threadIdx.x;
    if (i >= nc) return;
    const GBox bi = sb[threadIdx.x + kPlocRadius];
    float best = __int_as_float(0x7f800000);
    int bj = -1;
    const int lo = max(0, i - kPlocRadius), hi = min(nc - 1, i + kPlocRadius);
    for (int j = lo; j <= hi; j++) {
        if (j == i) continue;
        float a = box_area(box_union(bi, sb[j - b0 + kPlocRadius]));
        if (!(a == a)) a = __int_as_float(0x7f800000);  // a box with NaN coordinates: farthest
        if (bj < 0 || a < best) {  // ascending j: an equal area keeps the lower position
            best = a;
            bj = j;
        }
    }
    nearest[i] = bj;
}

// mutual nearest neighbours merge (the lower position creates the node and takes its place; the
// higher one leaves); everything else stays.  keep[i] = 1 for the clusters of the next round.
__global__ void k_ploc_merge(const int32_t* __restrict__ cluster, int nc, const int32_t* __restrict__ nearest,
                             GBox* __restrict__ box, int32_t* __restrict__ size, int32_t* __restrict__ left,
                             int32_t* __restrict__ right, int32_t* __restrict__ parent, uint32_t* __restrict__ next_id,
                             int32_t* __restrict__ merged, uint8_t* __restrict__ keep, int max_internal,
                             uint32_t* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const int j = nearest[i];
    const bool mutual = j >= 0 && nearest[j] == i;
    if (!mutual) {
        merged[i] = cluster[i];
        keep[i] = 1;
        return;
    }
    if (i > j) {
        keep[i] = 0;
        return;
    }
    const uint32_t id = atomicAdd(next_id, 1u);
    if ((int)id >= max_internal) {  // cannot happen for a consistent clustering; never write past
        atomicOr(err, 2u);
        keep[i] = 0;
        return;
    }
    const int a = cluster[i], b = cluster[j];
    left[id] = a;
    right[id] = b;
    parent[a] = (int32_t)id;
    parent[b] = (int32_t)id;
    box[id] = box_union(box[a], box[b]);
    size[id] = size[a] + size[b];
    merged[i] = (int32_t)id;
    keep[i] = 1;
}

// does ordering `face` put the canonical first child (a) first? (bvh.cpp:287-301)
__device__ __forceinline__ bool keep_order(int face, const GBox& a, const GBox& b) {
    switch (face) {
        case 0: return true;
        case 1: return a.mx[0] > b.mx[0];
        case 2: return a.mn[1] < b.mn[1];
        case 3: return a.mx[1] > b.mx[1];
        case 4: return a.mn[2] < b.mn[2];
        default: return a.mx[2] > b.mx[2];
    }
}

// preorder position of every node in all six orderings, and the output arrays
__global__ void k_orderings(int n, const uint32_t* __restrict__ sorted_tri, const int32_t* __restrict__ left,
                            const int32_t* __restrict__ right, const int32_t* __restrict__ parent,
                            const GBox* __restrict__ box, const int32_t* __restrict__ size,
                            float* __restrict__ node_bounds, int32_t* __restrict__ node_triangle,
                            int32_t* __restrict__ order_base, int32_t* __restrict__ order_miss,
                            uint32_t* __restrict__ err) {
    const int nn = 2 * n - 1;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nn) return;
    int pos[6] = {0, 0, 0, 0, 0, 0};
    int c = x;
    for (int steps = 0;; steps++) {
        const int p = parent[c];
        if (p < 0) break;
        if (steps > nn) {  // bounded: a valid tree is shallower than its node count
            atomicOr(err, 1u);
            return;
        }
        const int l = left[p], r = right[p];
        // canonical order: smaller min.x first (bvh.cpp:159-168)
        const bool l_first = box[l].mn[0] < box[r].mn[0];
        const int a = l_first ? l : r, b = l_first ? r : l;  // canonical first, second
        const GBox ba = box[a], bb = box[b];
        for (int f = 0; f < 6; f++) {
            const bool keep = keep_order(f, ba, bb);
            const int first = keep ? a : b;
            pos[f] += 1 + (c == first ? 0 : 2 * size[first] - 1);  // nodes of the preceding subtree
        }
        c = p;
    }
    const bool leaf = x >= n - 1;
    const int canon = pos[0];
    const GBox bx = box[x];
    for (int k = 0; k < 3; k++) {
        node_bounds[(size_t)canon * 6 + k] = bx.mn[k];
        node_bounds[(size_t)canon * 6 + 3 + k] = bx.mx[k];
    }
    node_triangle[canon] = leaf ? (int32_t)sorted_tri[x - (n - 1)] : -1;
    const int sub = 2 * size[x] - 1;  // nodes in x's subtree (size counts its leaves)
    for (int f = 0; f < 6; f++) {
        const int q = pos[f];
        order_base[(size_t)f * nn + q] = canon;
        order_miss[(size_t)f * nn + q] = leaf ? q + 1 : (q + sub < nn ? q + sub : -1);
    }
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, sizeof(T) * (n ? n : 1)); }
};

}  // namespace

namespace {

int build_gpu(sppm_mesh* m, int device, int builder) {
    if (!m) return fail(SPPM_ERR_ARG, "sppm_mesh_build_bvh_gpu: null mesh");
    if (builder != SPPM_BVH_GPU_PLOC && builder != SPPM_BVH_GPU_LBVH)
        return fail(SPPM_ERR_ARG, "sppm_mesh_build_bvh_gpu_ex: unknown builder %d", builder);
    const int n = (int)m->num_triangles;
    if (n < 1) return fail(SPPM_ERR_ARG, "sppm_mesh_build_bvh_gpu: mesh has no triangles");
    if (n > (1 << 28)) return fail(SPPM_ERR_ARG, "sppm_mesh_build_bvh_gpu: more than 2^28 triangles");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SPPM_ERR_NO_DEVICE, "no CUDA device is visible");
    }
    if (device < 0 || device >= ndev) return fail(SPPM_ERR_ARG, "device %d out of range", device);
    SPPM_CK(cudaSetDevice(device));
    const int nn = 2 * n - 1;
    std::vector<float> cen((size_t)n * 3);
    std::vector<GBox> tb(n);
    for (int i = 0; i < n; i++) {
        cen[(size_t)i * 3 + 0] = m->tri_centroid[i].x;
        cen[(size_t)i * 3 + 1] = m->tri_centroid[i].y;
        cen[(size_t)i * 3 + 2] = m->tri_centroid[i].z;
        const sppm::Box& b = m->tri_bbox[i];
        tb[i] = GBox{{b.mn.x, b.mn.y, b.mn.z}, {b.mx.x, b.mx.y, b.mx.z}};
    }
    DevBuf<float> d_cen, d_bounds;
    DevBuf<GBox> d_tb, d_box;
    DevBuf<uint32_t> d_code, d_code2, d_idx, d_idx2, d_arr, d_err, d_next;
    DevBuf<int32_t> d_left, d_right, d_parent, d_size, d_tri, d_base, d_miss, d_clu, d_clu2, d_near, d_nsel;
    DevBuf<uint8_t> d_keep;
    DevBuf<char> d_tmp, d_tmp2;
    cudaError_t e = cudaSuccess;
    auto A = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    A(d_cen.alloc((size_t)n * 3));
    A(d_tb.alloc(n));
    A(d_code.alloc(n));
    A(d_code2.alloc(n));
    A(d_idx.alloc(n));
    A(d_idx2.alloc(n));
    A(d_left.alloc(n));
    A(d_right.alloc(n));
    A(d_parent.alloc(nn));
    A(d_box.alloc(nn));
    A(d_size.alloc(nn));
    A(d_arr.alloc(n));
    A(d_err.alloc(1));
    A(d_bounds.alloc((size_t)nn * 6));
    A(d_tri.alloc(nn));
    A(d_base.alloc((size_t)6 * nn));
    A(d_miss.alloc((size_t)6 * nn));
    if (builder == SPPM_BVH_GPU_PLOC) {
        A(d_clu.alloc(n));
        A(d_clu2.alloc(n));
        A(d_near.alloc(n));
        A(d_keep.alloc(n));
        A(d_nsel.alloc(1));
        A(d_next.alloc(1));
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SPPM_ERR_OOM, "sppm_mesh_build_bvh_gpu: device allocation failed: %s", cudaGetErrorString(e));
    }
    A(cudaMemcpy(d_cen.p, cen.data(), cen.size() * 4, cudaMemcpyHostToDevice));
    A(cudaMemcpy(d_tb.p, tb.data(), tb.size() * sizeof(GBox), cudaMemcpyHostToDevice));
    A(cudaMemset(d_arr.p, 0, (size_t)n * 4));
    A(cudaMemset(d_err.p, 0, 4));
    A(cudaMemset(d_parent.p, 0xFF, (size_t)nn * 4));
    const sppm::Box& sb = m->bbox;
    const float3 lo = make_float3(sb.mn.x, sb.mn.y, sb.mn.z);
    auto inv = [](float a, float b) { return b > a ? 1.0f / (b - a) : 0.0f; };
    const float3 inv_ext = make_float3(inv(sb.mn.x, sb.mx.x), inv(sb.mn.y, sb.mx.y), inv(sb.mn.z, sb.mx.z));
    const int T = 256;
    const int gb = (n + T - 1) / T;
    if (e == cudaSuccess) k_morton<<<gb, T>>>(d_cen.p, (uint32_t)n, lo, inv_ext, d_code.p, d_idx.p);
    A(cudaGetLastError());
    size_t tmp_bytes = 0;
    A(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_code.p, d_code2.p, d_idx.p, d_idx2.p, n, 0, 30));
    A(d_tmp.alloc(tmp_bytes));
    A(cub::DeviceRadixSort::SortPairs(d_tmp.p, tmp_bytes, d_code.p, d_code2.p, d_idx.p, d_idx2.p, n, 0, 30));
    if (builder == SPPM_BVH_GPU_LBVH) {
        if (e == cudaSuccess && n > 1)
            k_radix_tree<<<(n - 1 + T - 1) / T, T>>>(d_code2.p, n, d_left.p, d_right.p, d_parent.p);
        A(cudaGetLastError());
        if (e == cudaSuccess)
            k_bounds<<<gb, T>>>(d_idx2.p, d_tb.p, n, d_left.p, d_right.p, d_parent.p, d_box.p, d_size.p, d_arr.p);
        A(cudaGetLastError());
    } else {
        if (e == cudaSuccess) k_ploc_leaves<<<gb, T>>>(d_idx2.p, d_tb.p, n, d_box.p, d_size.p, d_clu.p);
        A(cudaGetLastError());
        A(cudaMemset(d_next.p, 0, 4));
        size_t sel_bytes = 0;
        A(cub::DeviceSelect::Flagged(nullptr, sel_bytes, d_clu2.p, d_keep.p, d_clu.p, d_nsel.p, n));
        A(d_tmp2.alloc(sel_bytes));
        // every round merges at least the closest pair, so n - 1 rounds bound the loop
        int nc = n;
        for (int round = 0; nc > 1 && e == cudaSuccess; round++) {
            if (round >= n) {
                e = cudaErrorUnknown;
                return fail(SPPM_ERR_STATE, "sppm_mesh_build_bvh_gpu: clustering made no progress");
            }
            const int blocks = (nc + kPlocBlock - 1) / kPlocBlock;
            k_ploc_nearest<<<blocks, kPlocBlock>>>(d_clu.p, nc, d_box.p, d_near.p);
            k_ploc_merge<<<(nc + T - 1) / T, T>>>(d_clu.p, nc, d_near.p, d_box.p, d_size.p, d_left.p, d_right.p,
                                                  d_parent.p, d_next.p, d_clu2.p, d_keep.p, n - 1, d_err.p);
            A(cudaGetLastError());
            A(cub::DeviceSelect::Flagged(d_tmp2.p, sel_bytes, d_clu2.p, d_keep.p, d_clu.p, d_nsel.p, nc));
            int32_t left_count = 0;
            A(cudaMemcpy(&left_count, d_nsel.p, 4, cudaMemcpyDeviceToHost));
            if (e == cudaSuccess && (left_count < 1 || left_count >= nc)) {
                return fail(SPPM_ERR_STATE, "sppm_mesh_build_bvh_gpu: clustering round %d kept %d of %d clusters",
                            round, left_count, nc);
            }
            nc = left_count;
        }
        // the last cluster is the root
        int32_t root = 0;
        A(cudaMemcpy(&root, d_clu.p, 4, cudaMemcpyDeviceToHost));
        const int32_t none = -1;
        if (e == cudaSuccess && (root < 0 || root >= nn)) return fail(SPPM_ERR_STATE, "bad root %d", root);
        A(cudaMemcpy(d_parent.p + root, &none, 4, cudaMemcpyHostToDevice));
    }
    if (e == cudaSuccess)
        k_orderings<<<(nn + T - 1) / T, T>>>(n, d_idx2.p, d_left.p, d_right.p, d_parent.p, d_box.p, d_size.p,
                                             d_bounds.p, d_tri.p, d_base.p, d_miss.p, d_err.p);
    A(cudaGetLastError());
    A(cudaDeviceSynchronize());
    uint32_t err = 0;
    A(cudaMemcpy(&err, d_err.p, 4, cudaMemcpyDeviceToHost));
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "sppm_mesh_build_bvh_gpu: %s", cudaGetErrorString(e));
    if (err) return fail(SPPM_ERR_STATE, "sppm_mesh_build_bvh_gpu: inconsistent tree (%u)", err);
    m->num_nodes = (uint32_t)nn;
    m->node_bounds.resize((size_t)nn * 6);
    m->node_triangle.resize(nn);
    m->order_base.resize((size_t)6 * nn);
    m->order_miss.resize((size_t)6 * nn);
    A(cudaMemcpy(m->node_bounds.data(), d_bounds.p, (size_t)nn * 24, cudaMemcpyDeviceToHost));
    A(cudaMemcpy(m->node_triangle.data(), d_tri.p, (size_t)nn * 4, cudaMemcpyDeviceToHost));
    A(cudaMemcpy(m->order_base.data(), d_base.p, (size_t)6 * nn * 4, cudaMemcpyDeviceToHost));
    A(cudaMemcpy(m->order_miss.data(), d_miss.p, (size_t)6 * nn * 4, cudaMemcpyDeviceToHost));
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "sppm_mesh_build_bvh_gpu: %s", cudaGetErrorString(e));
    return SPPM_OK;
}

}  // namespace

extern "C" int sppm_mesh_build_bvh_gpu(sppm_mesh* m, int device) { return build_gpu(m, device, SPPM_BVH_GPU_PLOC); }

extern "C" int sppm_mesh_build_bvh_gpu_ex(sppm_mesh* m, int device, int builder) {
    return build_gpu(m, device, builder);
}

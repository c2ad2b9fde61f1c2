// GPU construction of the threaded BVH arrays (sppm_mesh_build_bvh_gpu): a linear BVH.
//
// The host builder (csrc/host/scene_bvh.cpp) reproduces the reference's exact-SAH tree node for
// node, which costs seconds per million triangles.  This builder makes a different tree in the
// same layout, in milliseconds:
//  1. 30-bit Morton code of each triangle centroid in the scene box; triangles sorted by
//     (code, index);
//  2. the radix tree over the sorted codes (Karras, "Maximizing parallelism in the construction
//     of BVHs, octrees, and k-d trees", HPG 2012): internal node i covers a key range found from
//     the longest common prefixes of its neighbours, its split is the first key whose prefix with
//     the range's first key is shorter than the range's common prefix; equal codes are told apart
//     by their position;
//  3. boxes and subtree sizes bottom-up (the second child to finish computes its parent);
//  4. the six threaded orderings of the reference's layout (bvh.cpp:159-168, 287-315): canonical
//     child order = smaller min.x first, orderings 1..5 keep that order only when the face's
//     predicate holds, nodes numbered in preorder; each node finds its preorder position by
//     walking to the root (position = sum over ancestors of 1 + the node count of the sibling
//     subtree that precedes it; a subtree of k leaves has 2k-1 nodes), and its miss link is the
//     node that follows its subtree.
// Triangle sorting uses cub::DeviceRadixSort (the CUDA toolkit's sort).
#include <cstdint>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
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

extern "C" int sppm_mesh_build_bvh_gpu(sppm_mesh* m, int device) {
    if (!m) return fail(SPPM_ERR_ARG, "sppm_mesh_build_bvh_gpu: null mesh");
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
    DevBuf<uint32_t> d_code, d_code2, d_idx, d_idx2, d_arr, d_err;
    DevBuf<int32_t> d_left, d_right, d_parent, d_size, d_tri, d_base, d_miss;
    DevBuf<char> d_tmp;
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
    if (e == cudaSuccess && n > 1) k_radix_tree<<<(n - 1 + T - 1) / T, T>>>(d_code2.p, n, d_left.p, d_right.p, d_parent.p);
    A(cudaGetLastError());
    if (e == cudaSuccess)
        k_bounds<<<gb, T>>>(d_idx2.p, d_tb.p, n, d_left.p, d_right.p, d_parent.p, d_box.p, d_size.p, d_arr.p);
    A(cudaGetLastError());
    if (e == cudaSuccess)
        k_orderings<<<(nn + T - 1) / T, T>>>(n, d_idx2.p, d_left.p, d_right.p, d_parent.p, d_box.p, d_size.p,
                                             d_bounds.p, d_tri.p, d_base.p, d_miss.p, d_err.p);
    A(cudaGetLastError());
    A(cudaDeviceSynchronize());
    uint32_t err = 0;
    A(cudaMemcpy(&err, d_err.p, 4, cudaMemcpyDeviceToHost));
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "sppm_mesh_build_bvh_gpu: %s", cudaGetErrorString(e));
    if (err) return fail(SPPM_ERR_STATE, "sppm_mesh_build_bvh_gpu: inconsistent radix tree");
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

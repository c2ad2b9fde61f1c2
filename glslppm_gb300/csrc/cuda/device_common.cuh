// Device-side data layout and exact single-precision helpers of the SPPM path.
//
// Layout in HBM (one render job = one scene + camera + progressive state; a batch launch covers
// many jobs through a job table and prefix sums of their work items):
//   scene   NodeX   [6 orderings][num_nodes]  32 B, in the traversal order of each ordering, so the
//                   "hit" successor of node i is i+1 and only the miss link is stored
//           TriIsect[num_tris]  48 B  v0, e0 = v1-v0, e1 = v2-v0 (the intersection test's operands)
//           TriShade[num_tris]  96 B  geometric normal + material, v0..v2, decoded shading normals
//           DevMaterial[num_mats] 32 B, light CDF + triangle table
//   pixels  float4 SoA: position, reflectance, normal, rng, (emission, N), (tau, R); int tri; float t
//   photons float4 SoA: position(+nrm.x), flux(+nrm.y), direction(+nrm.z), rng; int2 (tri, depth)
//   hash    uint32 winner[slots], uint32 count[slots]
//   grid    (SPPM_FLAG_PHOTON_GRID) uint2 key[photons]; per launch uint32 ofs[slots + 1] and
//           16-byte records[photons] in hash-slot order (photon_grid.cuh)
// float4 SoA keeps every per-item access a single coalesced 16-byte load or store.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sppm.h"
#include "sppm_fpmath.h"
#include "sppm_texture.h"

namespace sppm_dev {

constexpr int32_t kEmitterBit = 1 << 30;  // leaf triangle belongs to a light (skipped by photons)
constexpr int32_t kTriMask = kEmitterBit - 1;
constexpr uint32_t kEmptySlot = 0xFFFFFFFFu;

constexpr uint32_t kCellTable = 4096;  // cells per axis of the plain path's cell-bound table

constexpr uint32_t kErrWatchdogTraverse = 1u;
constexpr uint32_t kErrWatchdogLight = 2u;

struct __align__(32) NodeX {
    float bmin[3];
    int32_t miss;  // position in the same ordering, -1 = end
    float bmax[3];
    int32_t tri;   // -1 internal; leaf: triangle id, | kEmitterBit for lights
};
static_assert(sizeof(NodeX) == 32, "NodeX is one 32-byte sector");

// 32 bytes of read-only data in one 256-bit global load (sm_100 and later); p 32-byte aligned
__device__ __forceinline__ void ldg32(const void* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

struct __align__(16) DevMaterial {
    float color[3];
    float eta;
    int32_t brdf;
    float g;
    float pad[2];
};

// 4-wide quantised BVH node of the mixed path (host layout: csrc/host/scene_bvh4.h, 64 bytes):
// w[0] = origin xyz, exponent bytes x|y|z|count; w[1] = children; w[2] = qlo x,y,z, qhi x;
// w[3] = qhi y,z
struct __align__(32) Node4Dev {
    float4 w[4];
};

// the photon a hash slot keeps, as the mixed-path gather reads it (32 bytes):
// w0 = cell x|y (int16), cell z (int16) | count (uint16), offset x|y, offset z (unorm16)
// w1 = flux r|g, b (FP16, scaled), direction x|y, z (snorm16)
struct __align__(16) SlotRec {
    uint4 w0, w1;
};

struct DevScene {
    const NodeX* nodes;       // [6][num_nodes]
    const Node4Dev* nodes4;   // mixed path
    float flux_unscale, flux_unscale_inv;  // FP16 flux scale of the mixed path (light area * pi)
    const float4* tri_isect;  // [num_tris][3]
    const float4* tri_shade;  // [num_tris][6]
    const DevMaterial* mats;
    const float* light_cdf;
    const int32_t* light_tri;
    uint32_t num_nodes, num_tris, num_lights, num_mats;
    float light_area, light_stride;
    float bsphere[4];
    // material textures: null tri_tex when no texture coordinate of the scene is below 1e10 (no
    // lookups can happen); tex [layers][512][512] RGBA8, mat_layer [num_mats] (-1: magenta)
    const float2* tri_tex;     // [num_tris][3] texture coordinates T0, T1, T2
    const uint8_t* tex;
    const int32_t* mat_layer;
    float mat_rcp;             // MaterialNumRcp = 1 / num_mats
    // [6][num_tris]: each triangle's leaf position in the six threaded orderings -- the order in
    // which the exact walk meets it, so the 4-wide walk breaks ties at equal t the same way
    const int32_t* tri_rank;
};

struct DevPixels {
    float4 *pos, *refl, *nrm, *rng, *emi_n, *flux_r;
    int32_t* tri;
    float* t;
    // mixed precision statistics as double-float pairs (value = x + y, |y| <= ulp(x) / 2): N, R^2
    // and tau (3 per pixel), kept in FP32 arithmetic (GB300's FP64 rate is a small fraction of FP32)
    float2 *stat_n, *stat_r2, *stat_tau;
};

struct DevPhotons {
    float4 *pos, *flux, *dir, *rng;
    int2* hit;  // (triangle or -1, path depth)
};

// mutable per-job frame state (written by single threads between stages)
struct JobState {
    uint32_t frame;           // index of the frame in progress
    uint32_t frames_started;
    uint32_t eye_samples;
    uint32_t is_eye_frame;
    uint32_t xs[4];           // xorshift128 stream of the anti-aliasing offsets
    float aa[2];
    uint32_t bbmax_key[3], bbmin_key[3];  // order-preserving encodings for atomicMax/atomicMin
    float bbmin[3], bbmax[3];             // expanded grid bbox (BBMin/BBMax)
    float initial_radius, grid_scale, hash_scale1, r0;
    uint32_t emitted_frame;
    uint32_t segments_frame;
    float num_photons_f32;
    uint32_t err;
    unsigned long long num_photons, photon_segments, eye_segments;
    unsigned long long count_nodes, count_tris, count_segments;  // traversal counters (when enabled)
    unsigned long long coop_segments;  // photon segments traced one per warp
    uint32_t cell_table_n;    // valid entries per axis of JobDesc::cell_bounds (0: none yet)
};

struct JobDesc {
    DevScene scene;
    DevPixels px;
    DevPhotons ph;
    uint32_t* winner;
    uint32_t* count;
    SlotRec* slots;  // mixed path
    // plain path: c / GridScale + BBMin for the integer cell coordinates c of each axis
    // ([3][kCellTable]), the bounds of progressive.fs's in-cell test (:79-81), rebuilt after every
    // eye pass's grid (the same correctly rounded operations as the test's own)
    float* cell_bounds;
    uint2* grid_key;  // [P] counting-sort grid (SPPM_FLAG_PHOTON_GRID): each stored photon's
                      // (hash slot, rank among the slot's photons) of the current pass
    JobState* state;
    float* image;  // W*H*3 resolve target
    float cam_pos[3], cam_u[3], cam_v[3], cam_w[3];
    float cam_cx, cam_cy, cam_dist;
    uint32_t W, H, PW, PH, hash_num;
    uint32_t max_path, eye_interval, radius_rule, flags, precision;
    float alpha, footprint, focal, aperture, fixed_radius;
};

// Ray binning: a counting sort of the queued rays by (direction class, origin cell) so that the
// rays one warp fetches start close together and walk the same node ordering. 24 direction
// classes (cube face of the direction x the signs of its two minor components) x 8^3 origin
// cells of the scene's bounding cube, Morton-ordered.
constexpr uint32_t kRayDirClasses = 24;
constexpr uint32_t kRayCellBits = 3;
constexpr uint32_t kRayBins = kRayDirClasses << (3 * kRayCellBits);
// eye pixels whose path the exact eye pass defers to its block-wide pass per frame (beyond it
// the per-thread walk traces them)
constexpr uint32_t kEyeDeferred = 4096;

// ray queue of the wavefront photon pass: org.w holds the photon's global item index
struct RayQueue {
    float4* org;
    float4* dir;
    float4* hit;          // (triangle or -1 as int bits, barycentrics v, w, u)
    uint32_t* counters;   // [0] rays queued, [1] fetch head of the trace kernel, [2] rays set aside,
                          // [3] eye pixels deferred, [4] walks handed to the tail kernel,
                          // [7] frames since the ray bins were last reordered
    uint32_t capacity;
    uint32_t* slow;       // [capacity] queue indices of the rays traced one per warp
    uint32_t* tail_list;  // [capacity] queue indices of the walks the tail kernel finishes
    float4* tail_state;   // [capacity] their state: closest t, material, next node, steps
    // binning (all null when the rays are traced in queue order)
    uint2* key;           // [capacity] (bin, rank within the bin)
    uint32_t* bins;       // [kRayBins] counts, then exclusive offsets
    // the order the bins are traced in: bin_rank[ray_bin] = the bin's position (the key's first
    // word and the index into bins); bin_cost[position] = (node steps << 32) + rays, summed by the
    // traversal since the last reorder, which puts the bins of the longest mean walks first
    uint32_t* bin_rank;             // [kRayBins]
    unsigned long long* bin_cost;   // [kRayBins]
    uint32_t* perm;       // [capacity] queue index of the i-th ray in bin order
    uint32_t* eye_deferred;  // [kEyeDeferred] launch indices of the deferred eye pixels
    uint32_t refill_steps;   // traversal steps a warp takes between refills of its idle lanes
                             // (0: 32 for the exact walk, 8 for the 4-wide one)
    uint32_t tail_lanes;     // exact walk: once the queue is drained, a warp with at most this many
                             // walking lanes finishes them with the warp-cooperative walk (0: never)
};

// a finished walk's node steps into its bin's cost: the lanes that finished together add per bin
// with one pair of atomics (the rays of a warp mostly share a bin, and so do the warps working at
// the same time, so per-ray atomics would queue on a few addresses)
__device__ __forceinline__ void bin_cost_add(const RayQueue& q, uint32_t bin, uint32_t steps) {
    const unsigned same = __match_any_sync(__activemask(), bin);
    const uint32_t sum = __reduce_add_sync(same, steps);
    if ((int)(threadIdx.x & 31) == __ffs(same) - 1) {
        uint32_t* c = reinterpret_cast<uint32_t*>(q.bin_cost + bin);  // (steps << 32) + rays
        atomicAdd(c, (uint32_t)__popc(same));
        atomicAdd(c + 1, sum);
    }
}

// counting-sort photon grid of the jobs of a launch with SPPM_FLAG_PHOTON_GRID, rebuilt every
// pass: the records of job k's hash slot s are rec[ofs[b + s]] .. rec[ofs[b + s + 1] - 1], b = the
// job's first hash slot in the launch (the hash-slot launch set's prefix[k]); photon_grid.cuh has
// the record format and the cells
struct PhotonGrid {
    uint32_t* ofs;        // [hash slots of the launch + 1] exclusive prefix sums of the slot counts
    uint4* rec;           // [photon slots of the launch] 16-byte photon records in slot order
    uint32_t* tile_sums;  // [tiles of 2048 hash slots] their sums, then exclusive prefix sums
    uint32_t tiles;
    uint32_t rec_capacity;
    uint32_t shift;       // grid cells: the reference's split 2^shift times along each axis
};

// the work of one launch: items [prefix[k], prefix[k+1]) belong to jobs[job_ids[k]]; a launch
// covers the global items [first, total) (first > 0 for the later waves of the photon pass)
struct LaunchSet {
    const JobDesc* jobs;
    const uint32_t* job_ids;
    const uint32_t* prefix;
    uint32_t njobs;
    uint32_t total;
    uint32_t first;
};

__device__ __forceinline__ int find_job(const LaunchSet& ls, uint32_t g) {
    int lo = 0, hi = (int)ls.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&ls.prefix[mid]) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// three-input minimum / maximum (one instruction on sm_100+); like fminf/fmaxf a NaN operand is
// ignored, so fmax3(a, b, c) == fmaxf(fmaxf(a, b), c) for every input that can compare equal
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// ---- exact single-precision vector helpers (pinned evaluation order, never fused) ----------
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 xyz(float4 a) { return f3{a.x, a.y, a.z}; }
__device__ __forceinline__ float4 f4(f3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk(xadd(a.x, b.x), xadd(a.y, b.y), xadd(a.z, b.z)); }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk(xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)); }
__device__ __forceinline__ f3 mul(f3 a, f3 b) { return mk(xmul(a.x, b.x), xmul(a.y, b.y), xmul(a.z, b.z)); }
__device__ __forceinline__ f3 scl(f3 a, float s) { return mk(xmul(a.x, s), xmul(a.y, s), xmul(a.z, s)); }
__device__ __forceinline__ f3 neg(f3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return xadd(xadd(xmul(a.x, b.x), xmul(a.y, b.y)), xmul(a.z, b.z)); }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return mk(xsub(xmul(a.y, b.z), xmul(b.y, a.z)), xsub(xmul(a.z, b.x), xmul(b.z, a.x)),
              xsub(xmul(a.x, b.y), xmul(b.x, a.y)));
}
__device__ __forceinline__ float length(f3 a) { return xsqrt(dot(a, a)); }
__device__ __forceinline__ f3 normalize(f3 a) { return scl(a, xdiv(1.0f, xsqrt(dot(a, a)))); }
__device__ __forceinline__ f3 reflect(f3 i, f3 n) {
    const float d = xmul(2.0f, dot(n, i));
    return sub(i, scl(n, d));
}
__device__ __forceinline__ f3 refract(f3 i, f3 n, float eta) {
    const float d = dot(n, i);
    const float k = xsub(1.0f, xmul(xmul(eta, eta), xsub(1.0f, xmul(d, d))));
    if (k < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    return sub(scl(i, eta), scl(n, xadd(xmul(eta, d), xsqrt(k))));
}
__device__ __forceinline__ float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ float fractf(float x) { return xsub(x, floorf(x)); }

// ---- the triangle test of raytrace() (eyeraytrace.fs:200-243, photontrace.fs:196-236) --------
// Moller-Trumbore on the packed operands (a = v0 | e0.x, b = e0.yz | e1.xy, c.x = e1.z), every
// operation correctly rounded in the shaders' order, so a triangle's t, u, v and w are the same
// numbers wherever this is called (plain and mixed traversals alike).  Returns true when the
// triangle is hit at 0 <= t < tbest; cull: reject det <= 1e-10 (back faces of a first eye bounce).
// tri_hit_exact: the same test without the comparison against the closest hit so far.
__device__ __forceinline__ bool tri_hit_exact(const float4& a, const float4& b, const float4& c, f3 org, f3 dir,
                                              bool cull, float& tt, float& u, float& v, float& w) {
    const f3 v0 = mk(a.x, a.y, a.z), e0 = mk(a.w, b.x, b.y), e1 = mk(b.z, b.w, c.x);
    const f3 pv = cross(dir, e1);
    const float det = dot(e0, pv);
    if (cull && !(det > 1e-10f)) return false;
    const f3 tv = sub(org, v0);
    const f3 qv = cross(tv, e0);
    u = xdiv(dot(tv, pv), det);
    v = xdiv(dot(dir, qv), det);
    tt = xdiv(dot(e1, qv), det);
    w = xsub(xsub(1.0f, u), v);
    return u >= 0.0f && v >= 0.0f && tt >= 0.0f && w >= 0.0f;
}
__device__ __forceinline__ bool tri_test_exact(const float4& a, const float4& b, const float4& c, f3 org, f3 dir,
                                               bool cull, float tbest, float& tt, float& u, float& v, float& w) {
    return tri_hit_exact(a, b, c, org, dir, cull, tt, u, v, w) && tt < tbest;
}

// the ordering a ray walks: the cube face of its direction (major axis, ties x before y before z;
// the negative face when that component is < 0)
__device__ __forceinline__ int cube_face(f3 d) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    if (ax >= ay && ax >= az) return d.x < 0.0f ? 1 : 0;
    if (ay >= az) return d.y < 0.0f ? 3 : 2;
    return d.z < 0.0f ? 5 : 4;
}

// ---- GPURnd (eyeraytrace.fs:326-347) and the cell hash (hash.fs:21-48) ---------------------
// lane constants q, r, a, m and the single-precision 1/m, 1/q, m/2 the shaders derive from them
#define SPPM_RND_LANE(i, q, r, a, m, qinv, minv)                                                \
    {                                                                                            \
        const float beta = floorf(xmul(s[i], qinv));                                             \
        const float p = xsub(xmul(a, xsub(s[i], xmul(beta, q))), xmul(beta, r));                 \
        const float beta2 = xadd(xmul(signf(-p), 0.5f * (m)), 0.5f * (m));                       \
        s[i] = xadd(p, beta2);                                                                   \
        v[i] = xmul(s[i], minv);                                                                 \
    }

// one lane of the step: the new state in s[L], the lane's value in v[L]
template <int L>
__device__ __forceinline__ void schrage_lane(float s[4], float v[4]) {
    if (L == 0) SPPM_RND_LANE(0, 1225.0f, 1112.0f, 3423.0f, 4194287.0f, 8.163265302e-04f, 2.384195454e-07f)
    if (L == 1) SPPM_RND_LANE(1, 1585.0f, 367.0f, 2646.0f, 4194277.0f, 6.309148157e-04f, 2.384201139e-07f)
    if (L == 2) SPPM_RND_LANE(2, 2457.0f, 92.0f, 1707.0f, 4194191.0f, 4.070004215e-04f, 2.384250024e-07f)
    if (L == 3) SPPM_RND_LANE(3, 2098.0f, 265.0f, 1999.0f, 4194167.0f, 4.766444326e-04f, 2.384263666e-07f)
}
// the value of lane L for state x (the new state is not kept)
template <int L>
__device__ __forceinline__ float schrage_value(float x) {
    float s[4] = {x, x, x, x}, v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    schrage_lane<L>(s, v);
    return v[L];
}

__device__ __forceinline__ void schrage4(float s[4], float v[4]) {
    schrage_lane<0>(s, v);
    schrage_lane<1>(s, v);
    schrage_lane<2>(s, v);
    schrage_lane<3>(s, v);
}

__device__ __forceinline__ float gpu_rnd(float4& n) {
    float s[4] = {n.x, n.y, n.z, n.w}, v[4];
    schrage4(s, v);
    n = make_float4(s[0], s[1], s[2], s[3]);
    return fractf(xsub(xadd(xsub(v[0], v[1]), v[2]), v[3]));
}

__device__ __forceinline__ uint32_t hash_cell(f3 cell, float grid_scale, float hash_scale1, float hash_num) {
    float s[4] = {xmul(cell.x, hash_scale1), xmul(cell.y, hash_scale1), xmul(cell.z, hash_scale1),
                  xmul(xmul(grid_scale, 0.5f), hash_scale1)};
    float v[4];
    schrage4(s, v);
    float h = floorf(xmul(fractf(xsub(xadd(xsub(v[0], v[1]), v[2]), v[3])), hash_num));
    if (!(h >= 0.0f)) h = 0.0f;
    const float hmax = xsub(hash_num, 1.0f);
    if (h > hmax) h = hmax;
    return (uint32_t)h;
}

// the slots of the 2x2x2 cells from `base` (cell c = base + (c & 1, c >> 1 & 1, c >> 2)): each hash
// lane depends on one coordinate (lane 3 on the grid scale alone), so the 32 lane steps of eight
// hash_cell calls reduce to seven; the combination per cell is hash_cell's
__device__ __forceinline__ void hash_cells8(f3 base, float grid_scale, float hash_scale1, float hash_num,
                                            uint32_t slot[8]) {
    // the coordinates as the callers form them (base + 0 turns -0 into +0)
    const float x0 = __fadd_rn(base.x, 0.0f), y0 = __fadd_rn(base.y, 0.0f), z0 = __fadd_rn(base.z, 0.0f);
    const float x1 = __fadd_rn(base.x, 1.0f), y1 = __fadd_rn(base.y, 1.0f), z1 = __fadd_rn(base.z, 1.0f);
    const float vx[2] = {schrage_value<0>(__fmul_rn(x0, hash_scale1)), schrage_value<0>(__fmul_rn(x1, hash_scale1))};
    const float vy[2] = {schrage_value<1>(__fmul_rn(y0, hash_scale1)), schrage_value<1>(__fmul_rn(y1, hash_scale1))};
    const float vz[2] = {schrage_value<2>(__fmul_rn(z0, hash_scale1)), schrage_value<2>(__fmul_rn(z1, hash_scale1))};
    const float vw = schrage_value<3>(__fmul_rn(__fmul_rn(grid_scale, 0.5f), hash_scale1));
    const float hmax = __fsub_rn(hash_num, 1.0f);
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const float u = __fsub_rn(__fadd_rn(__fsub_rn(vx[c & 1], vy[(c >> 1) & 1]), vz[c >> 2]), vw);
        float h = floorf(__fmul_rn(__fsub_rn(u, floorf(u)), hash_num));
        if (!(h >= 0.0f)) h = 0.0f;
        if (h > hmax) h = hmax;
        slot[c] = (uint32_t)h;
    }
}

// order-preserving float <-> uint32 encoding (for atomicMin/atomicMax on floats)
__device__ __forceinline__ uint32_t float_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

}  // namespace sppm_dev

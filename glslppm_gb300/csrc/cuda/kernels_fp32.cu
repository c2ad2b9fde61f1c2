// Plain-FP32 SPPM kernels for sm_103a: every operation of the reference shaders in IEEE single
// precision, in the order the shaders write it (see device_common.cuh for the pinned helpers),
// so each per-pixel and per-photon value is bit-identical to the CPU restatement.  This
// translation unit is also compiled with -fmad=false.
//
// One SPPM frame (m_display, glslppm.cpp:214-536) is one launch per stage over all jobs of a
// batch:
//   k_frame_begin        hash-slot clear + per-job frame bookkeeping (AA offset of the eye pass)
//   k_eye                eyeraytrace.fs, fused with the max/min reductions (warp shuffles + one
//                        atomic per warp) that replace ReduceTexture's 2x2 passes and 18 readbacks
//   k_grid               InitialRadius / grid (glslppm.cpp:294-311), on the device
//   k_photon_gen         photontrace.fs emission / bounce / Russian roulette + the sum reduction;
//                        queues each live photon's ray (with its bin for the counting sort)
//   k_ray_bins_*         counting sort of the queued rays by direction class and origin cell
//   k_trace_photons      persistent traversal of the queued rays (dynamic fetch); rays with a zero
//                        direction component are set aside for k_trace_photons_coop (one warp each)
//   k_photon_store       store rule + hash.fs + scatter.vs (depth test = atomicMin of the photon
//                        index) + correction.vs (additive blend = atomicAdd), warp-aggregated
//   k_gather             progressive.fs
//   k_resolve            re.fs (on demand)
// k_photon is the single-kernel form of gen + trace + store (SPPM_FLAG_FUSED_PHOTON).
#include <cstdint>

#include "bvh4_trace.cuh"
#include "device_common.cuh"
#include "kernels.h"
#include "photon_grid.cuh"

namespace sppm_dev {

// ----------------------------------------------------------------------------------------------
// traversal: the threaded BVH walk of raytrace() (eyeraytrace.fs:67-290, photontrace.fs:123-255)
// ----------------------------------------------------------------------------------------------
struct Hit {
    float t;
    int32_t tri;
    int32_t mat;
    float bu, bv, bw;  // Barycentric = (v, w, u)
};

// bin of a queued ray: direction class (cube face x signs of the two minor components) and the
// Morton index of its origin's cell in a grid over the scene's bounding cube
__device__ __forceinline__ uint32_t spread_bits4(uint32_t v) {  // bits 0..3 -> 0, 3, 6, 9
    v = (v | (v << 4)) & 0x0C3u;
    return (v | (v << 2)) & 0x249u;
}
__device__ __forceinline__ uint32_t ray_bin(const DevScene& s, f3 o, f3 d) {
    const float* bs = s.bsphere;
    const float half = (float)(1u << (kRayCellBits - 1));
    const float sc = half / fmaxf(bs[3], 1e-30f);
    const float top = 2.0f * half - 1.0f;
    const uint32_t cx = (uint32_t)fminf(fmaxf((o.x - bs[0]) * sc + half, 0.0f), top);
    const uint32_t cy = (uint32_t)fminf(fmaxf((o.y - bs[1]) * sc + half, 0.0f), top);
    const uint32_t cz = (uint32_t)fminf(fmaxf((o.z - bs[2]) * sc + half, 0.0f), top);
    const int face = cube_face(d);
    const int axis = face >> 1;
    const float m1 = axis == 0 ? d.y : d.x, m2 = axis == 2 ? d.y : d.z;
    const uint32_t cls = (uint32_t)face * 4u + (m1 < 0.0f ? 2u : 0u) + (m2 < 0.0f ? 1u : 0u);
    return (cls << (3 * kRayCellBits)) | (spread_bits4(cx) << 2) | (spread_bits4(cy) << 1) | spread_bits4(cz);
}

struct TraversalCount {
    uint32_t nodes = 0, tris = 0;
};

template <bool PHOTON, bool COUNT = false>
__device__ __forceinline__ Hit trace_exact(const DevScene& s, f3 org, f3 dir, bool cull, uint32_t& err,
                                           TraversalCount* cnt = nullptr) {
    Hit h;
    h.t = PHOTON ? 1.0e30f : 1.0e20f;
    h.tri = -1;
    h.mat = -1;
    h.bu = h.bv = h.bw = 0.0f;
    const NodeX* nodes = s.nodes + (size_t)cube_face(dir) * s.num_nodes;
    const f3 rcp = mk(xdiv(1.0f, dir.x), xdiv(1.0f, dir.y), xdiv(1.0f, dir.z));
    const f3 t0 = mul(neg(rcp), org);
    const int32_t nn = (int32_t)s.num_nodes;
    int32_t i = 0;
    for (int32_t steps = 0;; steps++) {
        if (steps > nn) {
            err |= kErrWatchdogTraverse;
            break;
        }
        float4 A, B;
        ldg32(nodes + i, A, B);
        if (COUNT) cnt->nodes++;
        const float lx = xadd(xmul(rcp.x, A.x), t0.x), ly = xadd(xmul(rcp.y, A.y), t0.y), lz = xadd(xmul(rcp.z, A.z), t0.z);
        const float hx = xadd(xmul(rcp.x, B.x), t0.x), hy = xadd(xmul(rcp.y, B.y), t0.y), hz = xadd(xmul(rcp.z, B.z), t0.z);
        const float tmin = fmax3(fminf(lx, hx), fminf(ly, hy), fminf(lz, hz));
        const float tmax = fmin3(fmaxf(lx, hx), fmaxf(ly, hy), fmaxf(lz, hz));
        const bool hit = (tmin <= tmax) && (tmin <= h.t) && (tmax >= 0.0f);
        const int32_t tri = __float_as_int(B.w);
        if (hit && tri >= 0 && (!PHOTON || !(tri & kEmitterBit))) {
            const int32_t t = tri & kTriMask;
            if (COUNT) cnt->tris++;
            const float4 a = __ldg(&s.tri_isect[(size_t)t * 3 + 0]);
            const float4 b = __ldg(&s.tri_isect[(size_t)t * 3 + 1]);
            const float4 c = __ldg(&s.tri_isect[(size_t)t * 3 + 2]);
            float tt, u, v, w;
            if (tri_test_exact(a, b, c, org, dir, !PHOTON && cull, h.t, tt, u, v, w)) {
                h.t = tt;
                h.tri = t;
                h.mat = __float_as_int(c.y);
                h.bu = v;
                h.bv = w;
                h.bw = u;
            }
        }
        const int32_t next = hit ? i + 1 : __float_as_int(A.w);
        if (next < 0 || next >= nn) break;
        i = next;
    }
    return h;
}

// A ray with a zero (or denormal-small) direction component has an infinite reciprocal, and
// 0 * inf or inf - inf turn that axis' slab into NaN, which fminf/fmaxf then ignore: the box test
// passes for every box the other axes allow (for a photon leaving the light straight down,
// every box), and the walk visits nearly the whole tree.  Such rays are rare (a few per 10^7)
// but each costs thousands of dependent node fetches, so they are traced by coop_trace_exact.
__device__ __forceinline__ bool slab_degenerate(f3 d) {
    return fabsf(d.x) < 1e-30f || fabsf(d.y) < 1e-30f || fabsf(d.z) < 1e-30f;
}

// Warp-cooperative form of trace_exact for one ray (all 32 lanes call it with the same
// arguments and get the same result).  The lanes evaluate the box and triangle tests of 32
// consecutive nodes at once; the walk itself -- which nodes are visited, in which order, and
// which triangle hit replaces the current one -- is then resolved with ballots in exactly the
// order of the scalar loop, so the result is the same bit for bit.  A node is visited as a hit
// when its box passes with the t of the closest hit so far; a visited leaf replaces the closest
// hit when its triangle test passes with that t; the walk goes to node + 1 after a hit and to
// the miss link otherwise.
// The walk may also be resumed where a scalar walk stopped: at node `start` with the closest hit
// `h0` after `steps0` steps (coop_trace_exact_from); the result is the scalar walk's all the same.
template <bool PHOTON, bool COUNT>
__device__ __forceinline__ Hit coop_trace_exact_from(const DevScene& s, f3 org, f3 dir, bool cull, uint32_t& err,
                                                  TraversalCount* cnt, int32_t start, Hit h0, uint32_t steps0) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const int lane = (int)(threadIdx.x & 31);
    Hit h = h0;
    const NodeX* nodes = s.nodes + (size_t)cube_face(dir) * s.num_nodes;
    const f3 rcp = mk(xdiv(1.0f, dir.x), xdiv(1.0f, dir.y), xdiv(1.0f, dir.z));
    const f3 t0 = mul(neg(rcp), org);
    const int32_t nn = (int32_t)s.num_nodes;
    int32_t cur = start;
    uint32_t steps = steps0;
    bool done = start < 0 || start >= nn;
    while (!done) {
        const int32_t base = cur;
        const int32_t j = base + lane;
        bool box = false, leaf = false, ok = false;
        float tmin = 0.0f, tt = 0.0f, bu = 0.0f, bv = 0.0f, bw = 0.0f;
        int32_t miss = -1, tri = -1, mat = -1;
        if (j < nn) {
            float4 A, B;
            ldg32(nodes + j, A, B);
            const float lx = xadd(xmul(rcp.x, A.x), t0.x), ly = xadd(xmul(rcp.y, A.y), t0.y), lz = xadd(xmul(rcp.z, A.z), t0.z);
            const float hx = xadd(xmul(rcp.x, B.x), t0.x), hy = xadd(xmul(rcp.y, B.y), t0.y), hz = xadd(xmul(rcp.z, B.z), t0.z);
            tmin = fmax3(fminf(lx, hx), fminf(ly, hy), fminf(lz, hz));
            const float tmax = fmin3(fmaxf(lx, hx), fmaxf(ly, hy), fmaxf(lz, hz));
            box = (tmin <= tmax) && (tmax >= 0.0f);
            miss = __float_as_int(A.w);
            const int32_t raw = __float_as_int(B.w);
            leaf = raw >= 0 && (!PHOTON || !(raw & kEmitterBit));
            if (leaf && box) {
                tri = raw & kTriMask;
                const float4 a = __ldg(&s.tri_isect[(size_t)tri * 3 + 0]);
                const float4 b = __ldg(&s.tri_isect[(size_t)tri * 3 + 1]);
                const float4 c = __ldg(&s.tri_isect[(size_t)tri * 3 + 2]);
                const f3 v0 = mk(a.x, a.y, a.z), e0 = mk(a.w, b.x, b.y), e1 = mk(b.z, b.w, c.x);
                const f3 pv = cross(dir, e1);
                const float det = dot(e0, pv);
                if (PHOTON || !cull || det > 1e-10f) {
                    const f3 tv = sub(org, v0);
                    const f3 qv = cross(tv, e0);
                    const float u = xdiv(dot(tv, pv), det);
                    const float v = xdiv(dot(dir, qv), det);
                    tt = xdiv(dot(e1, qv), det);
                    const float w = xsub(xsub(1.0f, u), v);
                    ok = u >= 0.0f && v >= 0.0f && tt >= 0.0f && w >= 0.0f;
                    mat = __float_as_int(c.y);
                    bu = v;
                    bv = w;
                    bw = u;
                }
            }
        }
        const unsigned inwin = __ballot_sync(kFull, j < nn);
        const unsigned leaves = __ballot_sync(kFull, leaf);
        int pos = 0;
        for (;;) {
            const unsigned ge = kFull << pos;
            const unsigned M = __ballot_sync(kFull, box && tmin <= h.t) & ge & inwin;  // hits with the current t
            const unsigned U = __ballot_sync(kFull, ok && tt < h.t) & M;               // hits that replace it
            const unsigned notM = ~M & ge;
            const int stop = notM ? __ffs(notM) - 1 : 32;  // first lane >= pos that is not a hit
            const unsigned run = (stop == 32 ? kFull : ((1u << stop) - 1u)) & ge;
            const unsigned ur = U & run;
            if (ur) {
                const int p = __ffs(ur) - 1;  // visits pos..p, the leaf at p replaces the hit
                const unsigned vis = run & (p == 31 ? kFull : ((2u << p) - 1u));
                steps += __popc(vis);
                if (COUNT) {
                    cnt->nodes += __popc(vis);
                    cnt->tris += __popc(vis & leaves);
                }
                h.t = __shfl_sync(kFull, tt, p);
                h.tri = __shfl_sync(kFull, tri, p);
                h.mat = __shfl_sync(kFull, mat, p);
                h.bu = __shfl_sync(kFull, bu, p);
                h.bv = __shfl_sync(kFull, bv, p);
                h.bw = __shfl_sync(kFull, bw, p);
                if (p == 31) {
                    cur = base + 32;
                    done = cur >= nn;
                    break;
                }
                pos = p + 1;
                if (base + pos >= nn) {
                    done = true;
                    break;
                }
                continue;
            }
            steps += __popc(run);  // pos..stop-1 visited as hits, none replaces the hit
            if (COUNT) {
                cnt->nodes += __popc(run);
                cnt->tris += __popc(run & leaves);
            }
            if (stop == 32) {
                cur = base + 32;
                done = cur >= nn;
                break;
            }
            if (!((inwin >> stop) & 1u)) {  // the walk stepped past the last node
                done = true;
                break;
            }
            steps += 1;  // lane `stop` is visited and missed: follow its miss link
            if (COUNT) cnt->nodes += 1;
            const int32_t nx = __shfl_sync(kFull, miss, stop);
            if (nx < 0 || nx >= nn) {
                done = true;
                break;
            }
            if (nx > base + stop && nx < base + 32) {
                pos = nx - base;
                continue;
            }
            cur = nx;
            break;
        }
        if (steps > (uint32_t)nn + 1u) {
            err |= kErrWatchdogTraverse;
            done = true;
        }
    }
    return h;
}

template <bool PHOTON, bool COUNT>
__device__ __forceinline__ Hit coop_trace_exact(const DevScene& s, f3 org, f3 dir, bool cull, uint32_t& err,
                                                TraversalCount* cnt) {
    Hit h;
    h.t = PHOTON ? 1.0e30f : 1.0e20f;
    h.tri = -1;
    h.mat = -1;
    h.bu = h.bv = h.bw = 0.0f;
    return coop_trace_exact_from<PHOTON, COUNT>(s, org, dir, cull, err, cnt, 0, h, 0u);
}

// Block-wide form of the same walk (1024 threads, one ray, the same result bit for bit): the
// threads evaluate the box and triangle tests of 1024 consecutive nodes into shared memory; one
// warp then resolves the walk with 32-bit masks of the window -- M = nodes whose box passes with
// the current closest t, U = those of M whose triangle would replace the closest hit -- jumping
// straight to the next "event" (first node at or after the walk's position that is not in M, or
// is in U).  All nodes before an event are visited as hits without effect, so a window costs a
// few mask operations per event instead of a step per node; M and U are recomputed only when the
// closest hit changes.
constexpr int kBlockWalk = 1024;
constexpr int kBlockWords = kBlockWalk / 32;

struct BlockWalkShared {
    float tmin[kBlockWalk], tt[kBlockWalk], bu[kBlockWalk], bv[kBlockWalk], bw[kBlockWalk];
    int32_t miss[kBlockWalk], tri[kBlockWalk], mat[kBlockWalk];
    uint32_t box[kBlockWords], leaf[kBlockWords], ok[kBlockWords], inwin[kBlockWords];
    uint32_t M[kBlockWords], U[kBlockWords];  // with the closest t at the window's start
    // the walk's state, broadcast to the block between windows
    Hit h;
    int32_t cur;
    uint32_t steps, nodes, tris;
    int done;
};

template <bool PHOTON, bool COUNT>
__device__ __noinline__ Hit block_trace_exact(const DevScene& s, f3 org, f3 dir, bool cull, uint32_t& err,
                                              TraversalCount* cnt, BlockWalkShared& sh) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const int t = (int)threadIdx.x;
    const int lane = t & 31;
    const NodeX* nodes = s.nodes + (size_t)cube_face(dir) * s.num_nodes;
    const f3 rcp = mk(xdiv(1.0f, dir.x), xdiv(1.0f, dir.y), xdiv(1.0f, dir.z));
    const f3 t0 = mul(neg(rcp), org);
    const int32_t nn = (int32_t)s.num_nodes;
    if (t == 0) {
        sh.h.t = PHOTON ? 1.0e30f : 1.0e20f;
        sh.h.tri = -1;
        sh.h.mat = -1;
        sh.h.bu = sh.h.bv = sh.h.bw = 0.0f;
        sh.cur = 0;
        sh.steps = sh.nodes = sh.tris = 0;
        sh.done = 0;
    }
    __syncthreads();
    while (!sh.done) {
        const int32_t base = sh.cur;
        // ---- evaluate the window's nodes (every thread one node) ----
        {
            const int32_t j = base + t;
            bool box = false, leaf = false, ok = false;
            float tmin = 0.0f, tt = 0.0f, bu = 0.0f, bv = 0.0f, bw = 0.0f;
            int32_t miss = -1, tri = -1, mat = -1;
            if (j < nn) {
                float4 A, B;
                // two 16-byte loads: this toolkit's ptxas fails on the 256-bit form in this function
                A = __ldg(reinterpret_cast<const float4*>(nodes + j));
                B = __ldg(reinterpret_cast<const float4*>(nodes + j) + 1);
                const float lx = xadd(xmul(rcp.x, A.x), t0.x), ly = xadd(xmul(rcp.y, A.y), t0.y), lz = xadd(xmul(rcp.z, A.z), t0.z);
                const float hx = xadd(xmul(rcp.x, B.x), t0.x), hy = xadd(xmul(rcp.y, B.y), t0.y), hz = xadd(xmul(rcp.z, B.z), t0.z);
                tmin = fmax3(fminf(lx, hx), fminf(ly, hy), fminf(lz, hz));
                const float tmax = fmin3(fmaxf(lx, hx), fmaxf(ly, hy), fmaxf(lz, hz));
                box = (tmin <= tmax) && (tmax >= 0.0f);
                miss = __float_as_int(A.w);
                const int32_t raw = __float_as_int(B.w);
                leaf = raw >= 0 && (!PHOTON || !(raw & kEmitterBit));
                if (leaf && box) {
                    tri = raw & kTriMask;
                    const float4 a = __ldg(&s.tri_isect[(size_t)tri * 3 + 0]);
                    const float4 b = __ldg(&s.tri_isect[(size_t)tri * 3 + 1]);
                    const float4 c = __ldg(&s.tri_isect[(size_t)tri * 3 + 2]);
                    const f3 v0 = mk(a.x, a.y, a.z), e0 = mk(a.w, b.x, b.y), e1 = mk(b.z, b.w, c.x);
                    const f3 pv = cross(dir, e1);
                    const float det = dot(e0, pv);
                    if (PHOTON || !cull || det > 1e-10f) {
                        const f3 tv = sub(org, v0);
                        const f3 qv = cross(tv, e0);
                        const float u = xdiv(dot(tv, pv), det);
                        const float v = xdiv(dot(dir, qv), det);
                        tt = xdiv(dot(e1, qv), det);
                        const float w = xsub(xsub(1.0f, u), v);
                        ok = u >= 0.0f && v >= 0.0f && tt >= 0.0f && w >= 0.0f;
                        mat = __float_as_int(c.y);
                        bu = v;
                        bv = w;
                        bw = u;
                    }
                }
            }
            sh.tmin[t] = tmin;
            sh.tt[t] = tt;
            sh.bu[t] = bu;
            sh.bv[t] = bv;
            sh.bw[t] = bw;
            sh.miss[t] = miss;
            sh.tri[t] = tri;
            sh.mat[t] = mat;
            const float ht = sh.h.t;
            const bool m = box && j < nn && tmin <= ht;
            const unsigned bx = __ballot_sync(kFull, box), lf = __ballot_sync(kFull, leaf),
                           okm = __ballot_sync(kFull, ok), in = __ballot_sync(kFull, j < nn),
                           mm = __ballot_sync(kFull, m), um = __ballot_sync(kFull, m && ok && tt < ht);
            if (lane == 0) {
                sh.box[t >> 5] = bx;
                sh.leaf[t >> 5] = lf;
                sh.ok[t >> 5] = okm;
                sh.inwin[t >> 5] = in;
                sh.M[t >> 5] = mm;
                sh.U[t >> 5] = um;
            }
        }
        __syncthreads();
        // ---- one warp resolves the walk through the window ----
        if (t < 32) {
            const int w = lane;  // this lane's 32-node word
            Hit h = sh.h;
            uint32_t steps = sh.steps, cn = 0, ct = 0;
            int32_t next_window = -1;
            bool done = false;
            // M and U of words from..31 for the current closest t: word k from node k*32 + lane of
            // every lane (conflict-free shared reads), kept by lane k
            auto masks = [&](uint32_t& M, uint32_t& U, int from) {
                for (int k = from; k < kBlockWords; k++) {
                    const int n = k * 32 + lane;
                    const bool in = (sh.inwin[k] >> lane) & 1u, bx = (sh.box[k] >> lane) & 1u;
                    const bool m = in && bx && sh.tmin[n] <= h.t;
                    const bool u = m && ((sh.ok[k] >> lane) & 1u) && sh.tt[n] < h.t;
                    const unsigned bm = __ballot_sync(kFull, m), bu = __ballot_sync(kFull, u);
                    if (lane == k) {
                        M = bm;
                        U = bu;
                    }
                }
            };
            uint32_t M = sh.M[w], U = sh.U[w];
            const uint32_t leafw = sh.leaf[w], inw = sh.inwin[w];
            int pos = 0;
            for (;;) {
                // nodes at or after pos in this lane's word
                const int pw = pos >> 5;
                const uint32_t ge = w < pw ? 0u : (w > pw ? kFull : (kFull << (pos & 31)));
                const uint32_t ev = (~M | U) & ge;
                const unsigned has = __ballot_sync(kFull, ev != 0u);
                int e = kBlockWalk;  // event position (window end when none)
                if (has) {
                    const int fw = __ffs(has) - 1;
                    const uint32_t evw = __shfl_sync(kFull, ev, fw);
                    e = fw * 32 + __ffs(evw) - 1;
                }
                // nodes pos .. e-1 are visited as hits that change nothing
                {
                    const uint32_t lo = ge;
                    const uint32_t hi = (e >> 5) > w ? kFull : ((e >> 5) < w ? 0u : ((1u << (e & 31)) - 1u));
                    const uint32_t vis = lo & hi;
                    const uint32_t nv = __reduce_add_sync(kFull, __popc(vis));
                    steps += nv;
                    if (COUNT) {
                        cn += nv;
                        ct += __reduce_add_sync(kFull, __popc(vis & leafw));
                    }
                }
                if (e == kBlockWalk) {  // ran off the window's end: continue at the next node
                    next_window = base + kBlockWalk;
                    done = next_window >= nn;
                    break;
                }
                const int ew = e >> 5, eb = e & 31;
                const bool e_in = (__shfl_sync(kFull, inw, ew) >> eb) & 1u;
                if (!e_in) {  // the walk stepped past the last node
                    done = true;
                    break;
                }
                const bool e_upd = (__shfl_sync(kFull, U, ew) >> eb) & 1u;
                steps += 1;
                if (COUNT) cn += 1;
                if (e_upd) {  // a hit whose triangle replaces the closest hit
                    if (COUNT) ct += 1;
                    h.t = sh.tt[e];
                    h.tri = sh.tri[e];
                    h.mat = sh.mat[e];
                    h.bu = sh.bu[e];
                    h.bv = sh.bv[e];
                    h.bw = sh.bw[e];
                    pos = e + 1;
                    if (base + pos >= nn) {
                        done = true;
                        break;
                    }
                    if (pos == kBlockWalk) {
                        next_window = base + kBlockWalk;
                        break;
                    }
                    masks(M, U, pos >> 5);
                    continue;
                }
                // a node whose box misses: follow its miss link
                const int32_t nx = sh.miss[e];
                if (nx < 0 || nx >= nn) {
                    done = true;
                    break;
                }
                if (nx > base + e && nx < base + kBlockWalk) {
                    pos = nx - base;
                    continue;
                }
                next_window = nx;
                break;
            }
            if (lane == 0) {
                sh.h = h;
                sh.steps = steps;
                if (COUNT) {
                    sh.nodes += cn;
                    sh.tris += ct;
                }
                sh.cur = next_window;
                sh.done = done || steps > (uint32_t)nn + 1u;
                if (steps > (uint32_t)nn + 1u) sh.steps = 0xFFFFFFFFu;
            }
        }
        __syncthreads();
    }
    const Hit out = sh.h;
    if (sh.steps == 0xFFFFFFFFu) err |= kErrWatchdogTraverse;
    if (COUNT) {
        cnt->nodes += sh.nodes;
        cnt->tris += sh.tris;
    }
    __syncthreads();  // the shared state is read by every thread before a next ray reuses it
    return out;
}

struct Shade {
    f3 pos, nrm, gnrm, col;
    int brdf;
    float eta, g;
};

// Result of raytrace() for a hit (eyeraytrace.fs:256-287)
__device__ __forceinline__ Shade shade_hit(const DevScene& s, const Hit& h) {
    const float4* ts = s.tri_shade + (size_t)h.tri * 6;
    const float4 r0 = __ldg(ts + 0), r1 = __ldg(ts + 1), r2 = __ldg(ts + 2);
    const float4 r3 = __ldg(ts + 3), r4 = __ldg(ts + 4), r5 = __ldg(ts + 5);
    const f3 V0 = mk(r1.x, r1.y, r1.z), V1 = mk(r1.w, r2.x, r2.y), V2 = mk(r2.z, r2.w, r3.x);
    const f3 N0 = mk(r3.y, r3.z, r3.w), N1 = mk(r4.x, r4.y, r4.z), N2 = mk(r4.w, r5.x, r5.y);
    Shade o;
    o.pos = add(add(scl(V2, h.bu), scl(V0, h.bv)), scl(V1, h.bw));
    o.nrm = normalize(add(add(scl(N2, h.bu), scl(N0, h.bv)), scl(N1, h.bw)));
    o.gnrm = mk(r0.x, r0.y, r0.z);
    const DevMaterial& m = s.mats[h.mat];
    o.col = mk(m.color[0], m.color[1], m.color[2]);
    o.brdf = m.brdf;
    o.eta = m.eta;
    o.g = m.g;
    return o;
}

// col *= texture3D(VolumeTextureTextures, vec3(tex, r)).rgb when |tex.x| < 1e10 (eyeraytrace.fs:
// 443-446, photontrace.fs:418-422, 562-565), tex = T2 * b0 + T0 * b1 + T1 * b2 of the triangle's
// texture coordinates (eyeraytrace.fs:280); sampling as include/sppm_texture.h pins it
__device__ __forceinline__ f3 textured(const DevScene& S, int32_t tri, float b0, float b1, float b2, float r, f3 col) {
    const float2 T0 = __ldg(&S.tri_tex[(size_t)tri * 3]), T1 = __ldg(&S.tri_tex[(size_t)tri * 3 + 1]),
                 T2 = __ldg(&S.tri_tex[(size_t)tri * 3 + 2]);
    const float tu = xadd(xadd(xmul(T2.x, b0), xmul(T0.x, b1)), xmul(T1.x, b2));
    const float tv = xadd(xadd(xmul(T2.y, b0), xmul(T0.y, b1)), xmul(T1.y, b2));
    if (!(fabsf(tu) < 1e+10f)) return col;
    float t[3];
    sppm_tex_sample(S.tex, S.mat_layer, S.num_mats, tu, tv, r, t);
    return mk(xmul(col.x, t[0]), xmul(col.y, t[1]), xmul(col.z, t[2]));
}

// a photon bounce's colour: the hit's barycentrics from the stored position (photontrace.fs:
// 521-545), then the texture at layer (material + 0.5 + 0.25) / materials (:562-565)
__device__ __forceinline__ f3 textured_bounce(const DevScene& S, int32_t tri, f3 ipos, int32_t mat, f3 icol) {
    const float4* ts = S.tri_shade + (size_t)tri * 6;
    const float4 r1 = __ldg(ts + 1), r2 = __ldg(ts + 2), r3 = __ldg(ts + 3);
    const f3 V0 = mk(r1.x, r1.y, r1.z), V1 = mk(r1.w, r2.x, r2.y), V2 = mk(r2.z, r2.w, r3.x);
    const float bx = length(cross(sub(V1, V0), sub(ipos, V0)));
    const float by = length(cross(sub(V2, V1), sub(ipos, V1)));
    const float bz = length(cross(sub(V0, V2), sub(ipos, V2)));
    const float bs = xadd(xadd(bx, by), bz);
    return textured(S, tri, xdiv(bx, bs), xdiv(by, bs), xdiv(bz, bs),
                    xmul(S.mat_rcp, xadd(xadd((float)mat, 0.5f), 0.25f)), icol);
}

// ----------------------------------------------------------------------------------------------
// BRDF helpers (eyeraytrace.fs:293-392, photontrace.fs:60-89, 258-280, 443-461)
// ----------------------------------------------------------------------------------------------
__device__ __forceinline__ f3 onb(f3 x, f3 n) {
    if (n.z < -0.9999999f) return sub(scl(n, x.y), mk(x.z, x.x, 0.0f));
    const float a = xdiv(1.0f, xadd(1.0f, n.z));
    const float b = xmul(xmul(-n.x, n.y), a);
    const f3 u = mk(xsub(1.0f, xmul(xmul(n.x, n.x), a)), b, -n.x);
    const f3 w = mk(b, xsub(1.0f, xmul(xmul(n.y, n.y), a)), -n.y);
    return add(add(scl(u, x.x), scl(n, x.y)), scl(w, x.z));
}

__device__ __forceinline__ float fresnel(f3 incom, f3 normal, float ii, float ie) {
    const float eta = xdiv(ii, ie);
    const float c1 = dot(incom, normal);
    float c2 = xsub(1.0f, xmul(xmul(eta, eta), xsub(1.0f, xmul(c1, c1))));
    if (c2 < 0.0f) return 1.0f;
    c2 = xsqrt(c2);
    const float rs = xdiv(xsub(xmul(ii, c1), xmul(ie, c2)), xadd(xmul(ii, c1), xmul(ie, c2)));
    const float rp = xdiv(xsub(xmul(ii, c2), xmul(ie, c1)), xadd(xmul(ii, c2), xmul(ie, c1)));
    return xmul(xadd(xmul(rs, rs), xmul(rp, rp)), 0.5f);
}

__device__ __forceinline__ f3 glossy_reflect(f3 d, f3 n, float g, float4& rndv) {
    const f3 r = normalize(add(scl(reflect(d, n), xsub(xsub(1.0f, g), g)), scl(n, xadd(g, g))));
    const float rnd1 = gpu_rnd(rndv);
    const float rnd2 = gpu_rnd(rndv);
    const float temp1 = xmul(6.283184f, rnd1);
    const float temp2_ = sppm_fpow(rnd2, g);
    const float temp2 = xsqrt(xsub(1.0f, xmul(temp2_, temp2_)));
    const f3 v = mk(xmul(sppm_fsin(temp1), temp2), temp2_, xmul(sppm_fcos(temp1), temp2));
    f3 result = normalize(onb(v, r));
    if (dot(result, n) < 0.0f) result = reflect(result, n);
    return result;
}

__device__ __forceinline__ uint32_t grid_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }

// ----------------------------------------------------------------------------------------------
// k_frame_begin: clear the hashed grid of every job; per-job bookkeeping by the job's slot 0
// ----------------------------------------------------------------------------------------------
__device__ __forceinline__ float xorshift_frand(uint32_t* s) {
    const uint32_t t = s[0] ^ (s[0] << 11);
    s[0] = s[1];
    s[1] = s[2];
    s[2] = s[3];
    s[3] = (s[3] ^ (s[3] >> 19)) ^ (t ^ (t >> 8));
    return xmul(__uint2float_rn(s[3]), 1.0f / 4294967295.0f);
}

__global__ void k_frame_begin(LaunchSet ls, RayQueue q) {
    const uint32_t g = grid_tid();
    if (g == 0 && q.counters) {
        q.counters[0] = 0;
        q.counters[1] = 0;
        q.counters[2] = 0;
        q.counters[3] = 0;
        q.counters[4] = 0;
        q.counters[7] += 1u;  // frames since the bins were last reordered
    }
    if (q.bins && g < kRayBins) q.bins[g] = 0u;
    if (g >= ls.total) return;
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    const uint32_t local = g - ls.prefix[k];
    J.winner[local] = kEmptySlot;
    J.count[local] = 0;
    if (local == 0) {
        JobState* st = J.state;
        const uint32_t f = st->frames_started;
        st->frame = f;
        st->frames_started = f + 1;
        st->emitted_frame = 0;
        st->segments_frame = 0;
        const uint32_t interval = J.eye_interval ? J.eye_interval : 1u;
        st->is_eye_frame = (f % interval) == 0;
        if (st->is_eye_frame) {
            // AAOffset (glslppm.cpp:276-277)
            st->aa[0] = xmul(xsub(xorshift_frand(st->xs), 0.5f), 1.25f);
            st->aa[1] = xmul(xsub(xorshift_frand(st->xs), 0.5f), 1.25f);
            st->eye_samples += 1;
            for (int c = 0; c < 3; c++) {
                st->bbmax_key[c] = 0u;           // below every float
                st->bbmin_key[c] = 0xFFFFFFFFu;  // above every float
            }
        }
    }
}

// the photon ray queue emptied for the next wave of the photon pass (the eye pass's deferred
// pixel count, counters[3], belongs to the eye branch running beside the waves and is kept)
__global__ void k_queue_reset(RayQueue q) {
    const uint32_t g = grid_tid();
    if (g == 0) {
        q.counters[0] = 0;
        q.counters[1] = 0;
        q.counters[2] = 0;
        q.counters[4] = 0;
    }
    if (q.bins && g < kRayBins) q.bins[g] = 0u;
}

// ----------------------------------------------------------------------------------------------
// k_eye: eyeraytrace.fs main (:396-554) + max/min reduction of the hit positions
// ----------------------------------------------------------------------------------------------
__device__ __forceinline__ void warp_bbox_atomics(JobState* st, f3 p, int job_k) {
    // lanes of the same job combine with warp reductions; the leader issues one atomic per
    // component; a NaN component is ignored, as fminf/fmaxf ignore it
    const unsigned mask = __match_any_sync(__activemask(), job_k);
    const float v[3] = {p.x, p.y, p.z};
    for (int c = 0; c < 3; c++) {
        const bool ok = v[c] == v[c];
        uint32_t kmx = ok ? float_key(v[c]) : 0u;
        uint32_t kmn = ok ? float_key(v[c]) : 0xFFFFFFFFu;
        kmx = __reduce_max_sync(mask, kmx);
        kmn = __reduce_min_sync(mask, kmn);
        if ((threadIdx.x & 31) == (__ffs(mask) - 1)) {
            atomicMax(&st->bbmax_key[c], kmx);
            atomicMin(&st->bbmin_key[c], kmn);
        }
    }
}

// eye rays of the mixed path walk the 4-wide quantised BVH (the material comes from the triangle)
__device__ __forceinline__ Hit trace_eye4(const DevScene& s, f3 org, f3 dir, bool cull, uint32_t& err) {
    const Hit4 h4 = trace4<false>(s.nodes4, s.tri_isect, org, dir, cull, 1.0e20f, err,
                                  s.tri_rank ? s.tri_rank + (size_t)cube_face(dir) * s.num_tris : nullptr);
    Hit h;
    h.t = h4.t;
    h.tri = h4.tri;
    h.mat = h4.tri >= 0 ? __float_as_int(__ldg(&s.tri_isect[(size_t)h4.tri * 3 + 2]).y) : -1;
    h.bu = h4.bu;
    h.bv = h4.bv;
    h.bw = h4.bw;
    return h;
}

// the eye path of one pixel (eyeraytrace.fs main :396-554) up to its outputs; `trace(org, dir,
// cull, hit)` finds the closest hit and may decline (returns false), which abandons the path
// without side effects so that it can be rerun from its stored state
struct EyeOut {
    f3 pos, col, nrm, rdir, emi;
    float4 rndv;
    Hit last;
    uint32_t segs;
};

// TEX: the launch may hold a job whose scene has texture coordinates (texture lookups compiled in)
template <bool TEX, class Trace>
__device__ __forceinline__ bool eye_path(const JobDesc& J, const JobState* st, uint32_t p, Trace&& trace, EyeOut& out) {
    const uint32_t px = p % J.W, py = p / J.W;
    const DevScene& S = J.scene;
    float4 rndv = J.px.rng[p];
    const float eps = 1e-5f;
    const f3 U = mk(J.cam_u[0], J.cam_u[1], J.cam_u[2]);
    const f3 V = mk(J.cam_v[0], J.cam_v[1], J.cam_v[2]);
    const f3 Wd = mk(J.cam_w[0], J.cam_w[1], J.cam_w[2]);
    const f3 CP = mk(J.cam_pos[0], J.cam_pos[1], J.cam_pos[2]);
    const float aax = st->aa[0], aay = st->aa[1];
    const float ppx = xsub(xadd(xadd((float)px, 0.5f), aax), J.cam_cx);
    const float ppy = xsub(xadd(xadd((float)py, 0.5f), aay), J.cam_cy);
    f3 rdir = normalize(add(add(scl(U, ppx), scl(V, ppy)), scl(Wd, J.cam_dist)));
    f3 rorg;
    const float filter = xmul(xsub(1.0f, xdiv(fabsf(aax), 1.5f)), xsub(1.0f, xdiv(fabsf(aay), 1.5f)));
    {
        const f3 fp = add(CP, scl(rdir, J.focal));
        const float radius = xmul(xsqrt(gpu_rnd(rndv)), J.aperture);
        const float theta = xmul(6.283184f, gpu_rnd(rndv));
        const f3 lens = add(CP, scl(add(scl(U, sppm_fcos(theta)), scl(V, sppm_fsin(theta))), radius));
        rdir = normalize(sub(fp, lens));
        rorg = lens;
    }
    f3 col = mk(filter, filter, filter);
    f3 nrm = mk(0, 0, 0), pos = mk(0, 0, 0), emi = mk(0, 0, 0);
    Hit last;
    last.tri = -1;
    last.t = 1.0e20f;
    uint32_t segs = 0;
    for (uint32_t j = 0; j < J.max_path; j++) {
        Hit h;
        if (!trace(rorg, rdir, j == 0, h)) return false;  // deferred to the block-wide pass
        last = h;
        segs++;
        if (h.tri < 0) {
            nrm = mk(0, 0, 0);
            if (S.light_area == 0.0f) emi = mul(mk(0.7f, 0.7f, 1.0f), col);
            break;
        }
        Shade i = shade_hit(S, h);
        pos = i.pos;
        nrm = i.nrm;
        if (TEX && S.tri_tex)
            i.col = textured(S, h.tri, h.bu, h.bv, h.bw, xmul(S.mat_rcp, xadd((float)h.mat, 0.5f)), i.col);
        if (i.brdf == -1) {
            nrm = mk(0, 0, 0);
            emi = mul(col, i.col);
            break;
        } else if (i.brdf == 0) {
            col = mul(col, i.col);
            break;
        } else if (i.brdf == 1 || i.brdf == 4) {
            rorg = add(pos, scl(i.gnrm, eps));
            if (i.brdf == 4) nrm = glossy_reflect(nrm, nrm, i.g, rndv);
            rdir = reflect(rdir, nrm);
            if (dot(rdir, i.gnrm) < 0.0f) rdir = neg(rdir);
            col = mul(col, i.col);
        } else if (i.brdf == 2 || i.brdf == 5) {
            if (i.brdf == 5) nrm = glossy_reflect(nrm, nrm, i.g, rndv);
            const float ln = dot(nrm, rdir);
            if (ln < 0.0f) {
                const float re = fresnel(neg(rdir), nrm, 1.0f, i.eta);
                if (gpu_rnd(rndv) < re) {
                    rorg = add(pos, scl(i.gnrm, eps));
                    rdir = reflect(rdir, nrm);
                    if (dot(rdir, i.gnrm) < 0.0f) rdir = neg(rdir);
                } else {
                    col = mul(col, i.col);
                    rorg = sub(pos, scl(i.gnrm, eps));
                    rdir = refract(rdir, nrm, xdiv(1.0f, i.eta));
                    if (dot(rdir, i.gnrm) > 0.0f) rdir = neg(rdir);
                }
            } else {
                const float re = fresnel(neg(rdir), neg(nrm), i.eta, 1.0f);
                col = mul(col, i.col);
                if (gpu_rnd(rndv) < re) {
                    rorg = sub(pos, scl(i.gnrm, eps));
                    rdir = reflect(rdir, neg(nrm));
                    if (dot(rdir, neg(i.gnrm)) < 0.0f) rdir = neg(rdir);
                } else {
                    rorg = add(pos, scl(i.gnrm, eps));
                    rdir = refract(rdir, neg(nrm), i.eta);
                    if (dot(rdir, neg(i.gnrm)) > 0.0f) rdir = neg(rdir);
                }
            }
        } else if (i.brdf == 3 || i.brdf == 6) {
            if (i.brdf == 6) nrm = glossy_reflect(nrm, nrm, i.g, rndv);
            const float re = fresnel(neg(rdir), nrm, 1.0f, i.eta);
            if (gpu_rnd(rndv) < re) {
                rorg = add(pos, scl(i.gnrm, eps));
                rdir = reflect(rdir, nrm);
                if (dot(rdir, i.gnrm) < 0.0f) rdir = neg(rdir);
            } else {
                col = mul(col, i.col);
                break;
            }
        }
    }
    out.pos = pos;
    out.col = col;
    out.nrm = nrm;
    out.rdir = rdir;
    out.emi = emi;
    out.rndv = rndv;
    out.last = last;
    out.segs = segs;
    return true;
}

// the pixel outputs of a finished eye path (the running emission mean of :543-545)
__device__ __forceinline__ void eye_write(const JobDesc& J, const JobState* st, uint32_t p, const EyeOut& o) {
    float4 qe = J.px.emi_n[p];
    const float a = xdiv(1.0f, (float)st->eye_samples);
    const float oma = xsub(1.0f, a);
    qe.x = xadd(xmul(qe.x, oma), xmul(o.emi.x, a));
    qe.y = xadd(xmul(qe.y, oma), xmul(o.emi.y, a));
    qe.z = xadd(xmul(qe.z, oma), xmul(o.emi.z, a));
    J.px.pos[p] = f4(o.pos, o.rdir.x);
    J.px.refl[p] = f4(o.col, o.rdir.y);
    J.px.nrm[p] = f4(o.nrm, o.rdir.z);
    J.px.rng[p] = o.rndv;
    J.px.tri[p] = o.last.tri;
    J.px.t[p] = o.last.t;
    J.px.emi_n[p] = qe;
}

// eye pass, one thread per pixel.  A ray with a zero direction component (slab_degenerate)
// would walk most of the tree in one lane: the exact path defers such pixels to k_eye_coop
// (their whole path is rerun there with block-wide walks); the mixed path's slab tests do not
// degenerate.
template <bool MIXED, bool TEX>
__global__ void __launch_bounds__(128) k_eye(LaunchSet ls, uint32_t* deferred_n, uint32_t* deferred,
                                                uint32_t deferred_cap) {
    const uint32_t g = grid_tid();
    if (g >= ls.total) return;
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    JobState* st = J.state;
    const uint32_t p = g - ls.prefix[k];
    uint32_t err = 0;
    EyeOut o;
    const bool done = eye_path<TEX>(J, st, p, [&](f3 org, f3 dir, bool cull, Hit& h) {
        if (MIXED) {
            h = trace_eye4(J.scene, org, dir, cull, err);
            return true;
        }
        if (slab_degenerate(dir)) {
            const uint32_t slot = atomicAdd(deferred_n, 1u);
            if (slot < deferred_cap) {
                deferred[slot] = g;
                return false;
            }
        }
        h = trace_exact<false>(J.scene, org, dir, cull, err);
        return true;
    }, o);
    if (done) eye_write(J, st, p, o);
    const f3 bpos = done ? o.pos : mk(__int_as_float(0x7FC00000), __int_as_float(0x7FC00000), __int_as_float(0x7FC00000));
    warp_bbox_atomics(st, bpos, k);  // a deferred pixel contributes nothing (NaN is ignored)
    // segment count and errors: one atomic per warp and job
    const unsigned mask = __match_any_sync(__activemask(), k);
    const uint32_t wsegs = __reduce_add_sync(mask, done ? o.segs : 0u);
    const uint32_t werr = __reduce_or_sync(mask, err);
    if ((threadIdx.x & 31) == (__ffs(mask) - 1)) {
        atomicAdd(&st->eye_segments, (unsigned long long)wsegs);
        if (werr) atomicOr(&st->err, werr);
    }
}

// the deferred pixels of k_eye<false>, one block of 1024 threads per pixel: every thread runs
// the same path (identical values), each trace is block_trace_exact, thread 0 writes
template <bool TEX>
__global__ void __launch_bounds__(kBlockWalk) k_eye_coop(LaunchSet ls, const uint32_t* deferred_n,
                                                         const uint32_t* deferred, uint32_t deferred_cap) {
    __shared__ BlockWalkShared sh;
    const uint32_t n = min(*deferred_n, deferred_cap);
    for (uint32_t w = blockIdx.x; w < n; w += gridDim.x) {
        const uint32_t g = deferred[w];
        const int k = find_job(ls, g);
        const JobDesc& J = ls.jobs[ls.job_ids[k]];
        JobState* st = J.state;
        const uint32_t p = g - ls.prefix[k];
        uint32_t err = 0;
        EyeOut o;
        eye_path<TEX>(J, st, p, [&](f3 org, f3 dir, bool cull, Hit& h) {
            TraversalCount ct;
            h = block_trace_exact<false, false>(J.scene, org, dir, cull, err, &ct, sh);
            return true;
        }, o);
        if (threadIdx.x == 0) {
            eye_write(J, st, p, o);
            const float v[3] = {o.pos.x, o.pos.y, o.pos.z};
            for (int c = 0; c < 3; c++) {
                if (!(v[c] == v[c])) continue;
                atomicMax(&st->bbmax_key[c], float_key(v[c]));
                atomicMin(&st->bbmin_key[c], float_key(v[c]));
            }
            atomicAdd(&st->eye_segments, (unsigned long long)o.segs);
            if (err) atomicOr(&st->err, err);
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------------------------------------
// k_grid: glslppm.cpp:292-311 for every job in an eye frame (one thread per job)
// ----------------------------------------------------------------------------------------------
__global__ void k_grid(const JobDesc* jobs, const uint32_t* job_ids, uint32_t njobs) {
    const uint32_t k = grid_tid();
    if (k >= njobs) return;
    const JobDesc& J = jobs[job_ids[k]];
    JobState* st = J.state;
    float mx[3], mn[3];
    for (int c = 0; c < 3; c++) {
        mx[c] = key_float(st->bbmax_key[c]);
        mn[c] = key_float(st->bbmin_key[c]);
    }
    float r0;
    if (J.radius_rule == SPPM_RADIUS_DIAGONAL) {
        r0 = J.fixed_radius;
    } else {
        float bbsize = 0.0f;
        for (int c = 0; c < 3; c++) bbsize = xadd(bbsize, xsub(mx[c], mn[c]));
        r0 = xmul(xdiv(xdiv(bbsize, 3.0f), (float)J.W), J.footprint);
    }
    st->initial_radius = r0;
    for (int c = 0; c < 3; c++) {
        st->bbmin[c] = xsub(mn[c], r0);
        st->bbmax[c] = xadd(mx[c], r0);
    }
    st->grid_scale = xdiv(0.5f, r0);
    st->hash_scale1 = xdiv(4194304.0f, st->grid_scale);
    if (st->frame == 0) st->r0 = r0;
}

// k_cell_bounds: the in-cell test's bounds (progressive.fs:79-81: cell / GridScale + BBMin, with the
// test's own correctly rounded division and addition) for every integer cell coordinate of the
// grid k_grid has just set, a block per job of the eye phase
__global__ void __launch_bounds__(256) k_cell_bounds(const JobDesc* jobs, const uint32_t* job_ids) {
    const JobDesc& J = jobs[job_ids[blockIdx.x]];
    if (!J.cell_bounds) return;
    JobState* st = J.state;
    const float G = st->grid_scale;
    uint32_t n = 0;
    for (int a = 0; a < 3; a++) {
        const float e = xmul(xsub(st->bbmax[a], st->bbmin[a]), G);  // cells along the axis
        const uint32_t na = e >= 0.0f && e < (float)kCellTable ? (uint32_t)e + 3u : kCellTable;
        n = max(n, na);
    }
    n = min(n, kCellTable);
    for (uint32_t i = threadIdx.x; i < 3 * n; i += blockDim.x) {
        const uint32_t a = i / n, c = i - a * n;
        J.cell_bounds[a * kCellTable + c] = xadd(xdiv((float)c, G), st->bbmin[a]);
    }
    if (threadIdx.x == 0) st->cell_table_n = n;
}

// ----------------------------------------------------------------------------------------------
// k_photon: photontrace.fs main (:464-720), sum.fs, hash.fs + scatter.vs + correction.vs
// ----------------------------------------------------------------------------------------------
// GenerateLightSourceSample (photontrace.fs:345-440) up to its cosine lobe: the origin, the flux and
// the lobe's normal (the lobe itself is cosine_lobe, drawn right after, shared with the bounces)
template <bool TEX>
__device__ __forceinline__ void light_sample(const JobDesc& J, float4& rndv, f3& flux, f3& lobe_n, f3& org,
                                             uint32_t& err) {
    const DevScene& S = J.scene;
    const float rnd = gpu_rnd(rndv);
    int low = 0;
    int high = (int)xadd(xdiv(1.0f, S.light_stride), 0.5f);
    const int nl = (int)S.num_lights;
    // texel of search step `mid` at texcoord (mid - 0.5)*stride: index mid-1, clamped
    int guard = 0;
    while (low < high) {
        if (++guard > 64) {
            err |= kErrWatchdogLight;
            break;
        }
        const int mid = low + ((high - low) / 2);
        const int kk = min(max(mid - 1, 0), nl - 1);
        if (__ldg(&S.light_cdf[kk]) < rnd) low = mid + 1;
        else high = mid;
    }
    const int32_t lt = __ldg(&S.light_tri[min(max(high - 1, 0), nl - 1)]);
    const float rndv2 = gpu_rnd(rndv);
    const float t = xsqrt(xsub(1.0f, rndv2));
    const float sv = gpu_rnd(rndv);
    const float a = xsub(1.0f, t);
    const float c = xmul(sv, t);
    const float b = xsub(t, c);
    const float4* ts = S.tri_shade + (size_t)lt * 6;
    const float4 r0 = __ldg(ts + 0), r1 = __ldg(ts + 1), r2 = __ldg(ts + 2);
    const float4 r3 = __ldg(ts + 3), r4 = __ldg(ts + 4), r5 = __ldg(ts + 5);
    const f3 V0 = mk(r1.x, r1.y, r1.z), V1 = mk(r1.w, r2.x, r2.y), V2 = mk(r2.z, r2.w, r3.x);
    const f3 N0 = mk(r3.y, r3.z, r3.w), N1 = mk(r4.x, r4.y, r4.z), N2 = mk(r4.w, r5.x, r5.y);
    const DevMaterial& m = S.mats[__float_as_int(r0.w)];
    flux = scl(mk(m.color[0], m.color[1], m.color[2]), xmul(S.light_area, 3.141592f));
    if (TEX && S.tri_tex)  // T = T2 * c + T0 * a + T1 * b (photontrace.fs:413-422)
        flux = textured(S, lt, c, a, b, xmul(S.mat_rcp, xadd((float)__float_as_int(r0.w), 0.75f)), flux);
    f3 o = add(add(scl(V0, a), scl(V1, b)), scl(V2, c));
    const f3 nrm = normalize(add(add(scl(N0, a), scl(N1, b)), scl(N2, c)));
    const f3 gnrm = mk(r0.x, r0.y, r0.z);
    o = add(o, scl(gnrm, 1.0e-5f));
    lobe_n = nrm;
    org = o;
}

// cosine lobe around n (photontrace.fs:432-439 for emission, :567-578 for matte bounces): two draws
__device__ __forceinline__ f3 cosine_lobe(float4& rndv, f3 n) {
    const float r0 = xmul(6.283184f, gpu_rnd(rndv));
    const float r1 = xsqrt(gpu_rnd(rndv));
    return onb(mk(xmul(sppm_fsin(r0), r1), xsqrt(xsub(1.0f, xmul(r1, r1))), xmul(sppm_fcos(r0), r1)), n);
}

__device__ __forceinline__ void ibl_sample(const JobDesc& J, float4& rndv, f3& flux, f3& dir, f3& org) {
    const float* bs = J.scene.bsphere;
    const float area = xmul(xmul(12.566368f, bs[3]), bs[3]);
    const float temp2 = xmul(6.283184f, gpu_rnd(rndv));
    const float aaa = xsqrt(xsub(1.0f, gpu_rnd(rndv)));
    const float sinA = sppm_fsin(aaa);
    const float sinTemp1 = xmul(xadd(sinA, sinA), sppm_fcos(aaa));
    f3 d = mk(xmul(sinTemp1, sppm_fcos(temp2)), xsub(1.0f, xmul(xadd(sinA, sinA), sinA)), xmul(sinTemp1, sppm_fsin(temp2)));
    if (gpu_rnd(rndv) > 0.5f) {
        d = mk(1.0f, 1.0f, 1.0f);
        d.y = xadd(d.y, d.y);
        d.z = -d.z;
        d = normalize(d);
        flux = scl(mk(1.0f, 1.0f, 0.7f), area);
    } else {
        flux = scl(mk(0.7f, 0.7f, 1.0f), area);
    }
    const float radius = xsqrt(gpu_rnd(rndv));
    const float theta = xmul(6.283184f, gpu_rnd(rndv));
    const f3 temp = mk(xmul(radius, sppm_fcos(theta)), 0.0f, xmul(radius, sppm_fsin(theta)));
    org = add(add(onb(scl(temp, bs[3]), d), scl(d, bs[3])), mk(bs[0], bs[1], bs[2]));
    dir = neg(d);
}

// emit a photon or bounce the stored one (photontrace.fs main :464-686): the ray of this pass
struct PhotonRay {
    f3 org, dir, flux;
    float depth;
    bool cont;
    uint32_t emitted;
};

// hitin: the previous segment's (triangle, depth), (-1, 0) before the first; PP, PF, PD: its
// record (position, flux, direction, with the normal in the w components)
template <bool TEX>
__device__ __forceinline__ PhotonRay photon_generate(const JobDesc& J, int2 hitin, float4 PP, float4 PF, float4 PD,
                                                     float4& rndv, uint32_t& err) {
    // Emission and the diffuse bounces end in the same cosine lobe: each path sets up its lobe
    // (normal, origin; the draws before the lobe stay in the path) and the lanes draw the lobe
    // together, then finish their path (the flip against the geometric normal, Russian roulette).
    const DevScene& S = J.scene;
    const float eps = 1e-6f;
    PhotonRay R;
    R.org = mk(0, 0, 0);
    R.dir = mk(0, 0, 0);
    R.depth = xadd((float)hitin.y, 1.0f);
    const bool emit = hitin.x < 0 || R.depth >= (float)J.max_path;
    bool lobe = false, flip = false;
    f3 lobe_n = mk(0, 0, 0), gnrm = mk(0, 0, 0), icol = mk(0, 0, 0), flux = mk(0, 0, 0);
    f3 rorg = mk(0, 0, 0), rdir = mk(0, 0, 0);
    if (emit) {
        if (S.light_area != 0.0f) {
            light_sample<TEX>(J, rndv, R.flux, lobe_n, rorg, err);
            lobe = true;
        } else {
            ibl_sample(J, rndv, R.flux, rdir, rorg);
        }
    } else {
        flux = mk(fabsf(PF.x), fabsf(PF.y), fabsf(PF.z));
        const f3 ipos = xyz(PP);
        f3 inrm = mk(PP.w, PF.w, PD.w);
        const f3 pd = xyz(PD);
        const float4 r0 = __ldg(S.tri_shade + (size_t)hitin.x * 6);
        gnrm = mk(r0.x, r0.y, r0.z);
        const DevMaterial& m = S.mats[__float_as_int(r0.w)];
        icol = mk(m.color[0], m.color[1], m.color[2]);
        if (TEX && S.tri_tex) icol = textured_bounce(S, hitin.x, ipos, __float_as_int(r0.w), icol);
        const int brdf = m.brdf;
        if (brdf == 0) {
            rorg = add(ipos, scl(gnrm, eps));  // matte_bounce
            lobe_n = inrm;
            lobe = flip = true;
        } else if (brdf == 1 || brdf == 4) {
            rorg = add(ipos, scl(gnrm, eps));
            if (brdf == 4) inrm = glossy_reflect(inrm, inrm, m.g, rndv);
            rdir = reflect(pd, inrm);
            if (dot(rdir, gnrm) < 0.0f) rdir = neg(rdir);
        } else if (brdf == 2 || brdf == 5) {
            if (brdf == 5) inrm = glossy_reflect(inrm, inrm, m.g, rndv);
            const float ln = dot(inrm, pd);
            if (ln < 0.0f) {
                const float re = fresnel(neg(pd), inrm, 1.0f, m.eta);
                if (gpu_rnd(rndv) < re) {
                    rorg = add(ipos, scl(gnrm, eps));
                    rdir = reflect(pd, inrm);
                    icol = mk(1.0f, 1.0f, 1.0f);
                    if (dot(rdir, gnrm) < 0.0f) rdir = neg(rdir);
                } else {
                    rorg = sub(ipos, scl(gnrm, eps));
                    rdir = refract(pd, inrm, xdiv(1.0f, m.eta));
                    if (dot(rdir, gnrm) > 0.0f) rdir = neg(rdir);
                }
            } else {
                const float re = fresnel(neg(pd), neg(inrm), m.eta, 1.0f);
                if (gpu_rnd(rndv) < re) {
                    rorg = sub(ipos, scl(gnrm, eps));
                    rdir = reflect(pd, neg(inrm));
                    if (dot(rdir, neg(gnrm)) < 0.0f) rdir = neg(rdir);
                } else {
                    rorg = add(ipos, scl(gnrm, eps));
                    rdir = refract(pd, neg(inrm), m.eta);
                    if (dot(rdir, neg(gnrm)) > 0.0f) rdir = neg(rdir);
                }
            }
        } else if (brdf == 3 || brdf == 6) {
            if (brdf == 6) inrm = glossy_reflect(inrm, inrm, m.g, rndv);
            const float re = fresnel(neg(pd), inrm, 1.0f, m.eta);
            if (gpu_rnd(rndv) < re) {
                rorg = add(ipos, scl(gnrm, eps));
                rdir = reflect(pd, inrm);
                icol = mk(1.0f, 1.0f, 1.0f);
                if (dot(rdir, gnrm) < 0.0f) rdir = neg(rdir);
            } else {
                rorg = add(ipos, scl(gnrm, eps));  // matte_bounce
                lobe_n = inrm;
                lobe = flip = true;
            }
        }
    }
    if (lobe) {
        rdir = cosine_lobe(rndv, lobe_n);
        if (flip && dot(rdir, gnrm) < 0.0f) rdir = neg(rdir);
    }
    R.org = rorg;
    R.dir = rdir;
    if (emit) {
        R.emitted = 1;
        R.depth = 0.0f;
        R.cont = true;
        return R;
    }
    // Russian roulette (:671-685)
    const float pmax = fmaxf(fmaxf(icol.x, icol.y), icol.z);
    if (pmax < gpu_rnd(rndv)) {
        R.cont = false;
    } else {
        R.cont = true;
        icol = mk(xdiv(icol.x, pmax), xdiv(icol.y, pmax), xdiv(icol.z, pmax));
        flux = mul(flux, icol);
    }
    R.emitted = 0;
    R.flux = flux;
    return R;
}

template <bool TEX>
__device__ __forceinline__ PhotonRay photon_generate(const JobDesc& J, uint32_t sidx, uint32_t frame, float4& rndv,
                                                     uint32_t& err) {
    const int2 hitin = frame == 0 ? make_int2(-1, 0) : J.ph.hit[sidx];
    return photon_generate<TEX>(J, hitin, J.ph.pos[sidx], J.ph.flux[sidx], J.ph.dir[sidx], rndv, err);
}

__device__ __forceinline__ void photon_terminate(const JobDesc& J, uint32_t sidx) {
    J.ph.pos[sidx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    J.ph.flux[sidx] = make_float4(-1.0f, -1.0f, -1.0f, 0.0f);
    J.ph.dir[sidx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    J.ph.hit[sidx] = make_int2(-1, 0);
}

// store the traced photon (photontrace.fs :692-709); returns the hash slot or 0xFFFFFFFF
// (jobs with SPPM_FLAG_PHOTON_GRID: the slot of the counting-sort grid's cell, split grid_shift
// times, or 0xFFFFFFFF for a photon outside the grid)
__device__ __forceinline__ uint32_t photon_store(const JobDesc& J, const JobState* st, uint32_t sidx, const Hit& h,
                                                 f3 rdir, f3 flux, float depth, uint32_t grid_shift = 0) {
    const DevScene& S = J.scene;
    f3 ppos = mk(0, 0, 0), pnrm = mk(0, 0, 0), pg = mk(0, 0, 0);
    int brdf = 0;
    if (h.tri >= 0) {
        const Shade i = shade_hit(S, h);
        ppos = i.pos;
        pnrm = i.nrm;
        pg = i.gnrm;
        brdf = i.brdf;
    }
    if (h.tri < 0 || (brdf != 0 && brdf != 6 && brdf != 3)) flux = neg(flux);
    const float gf = fminf(fabsf(xdiv(dot(rdir, pnrm), dot(rdir, pg))), 2.236068010e+00f);
    flux = scl(flux, gf);
    J.ph.pos[sidx] = f4(ppos, pnrm.x);
    J.ph.flux[sidx] = f4(flux, pnrm.y);
    J.ph.dir[sidx] = f4(rdir, pnrm.z);
    J.ph.hit[sidx] = make_int2(h.tri, (int)depth);
    if (flux.x < 0.0f) return 0xFFFFFFFFu;
    if (J.flags & SPPM_FLAG_PHOTON_GRID) return grid_photon_slot(J, st, grid_shift, ppos.x, ppos.y, ppos.z);
    // hash.fs main (:51-68): cell = floor((p - BBoxMin) * GridScale), slot = hash(cell)
    const f3 cell = mk(floorf(xmul(xsub(ppos.x, st->bbmin[0]), st->grid_scale)),
                       floorf(xmul(xsub(ppos.y, st->bbmin[1]), st->grid_scale)),
                       floorf(xmul(xsub(ppos.z, st->bbmin[2]), st->grid_scale)));
    return hash_cell(cell, st->grid_scale, st->hash_scale1, (float)J.hash_num);
}

// scatter.vs + depth test and correction.vs + blend, one atomic pair per warp and slot
__device__ __forceinline__ void hash_insert(const JobDesc& J, int k, uint32_t sidx, uint32_t slot, unsigned active) {
    const bool store = slot != 0xFFFFFFFFu;
    // photon index order = depth order; photons of the last row with i >= w/2 have z >= 1 and are
    // clipped by the scatter draw (counted by the correction draw all the same).  A clipped photon
    // offers P (the photon count) to the minimum: a slot that only clipped photons reach keeps P,
    // which the gather reads as the cleared texel -- photon 0 -- weighted by the slot's count.
    const bool clipped = (J.flags & SPPM_FLAG_GL_DEPTH_CLIP) && sidx >= (J.PH - 1) * J.PW + (J.PW + 1) / 2;
    const unsigned long long key = store ? ((unsigned long long)k << 32) | slot : ~0ull;
    const unsigned peers = __match_any_sync(active, key);
    if (store) {
        const uint32_t n = __popc(peers);
        if (J.flags & SPPM_FLAG_PHOTON_GRID) {
            // counting-sort grid: the count, and each photon's rank among its slot's photons (the
            // order of the ranks within a slot is arbitrary: the gather's sums do not depend on it)
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(&J.count[slot], n);
            base = __shfl_sync(peers, base, leader);
            const uint32_t below = peers & ((1u << (threadIdx.x & 31)) - 1u);
            J.grid_key[sidx] = make_uint2(slot, base + __popc(below));
            return;
        }
        const uint32_t wmin = __reduce_min_sync(peers, clipped ? J.PW * J.PH : sidx);
        if ((threadIdx.x & 31) == (__ffs(peers) - 1)) {
            atomicAdd(&J.count[slot], n);
            if (wmin != 0xFFFFFFFFu) atomicMin(&J.winner[slot], wmin);
        }
    }
}

// sum.fs (emitted photons), traced segments and errors: one atomic per warp and job
__device__ __forceinline__ void photon_counters(JobState* st, int k, unsigned active, uint32_t emitted, uint32_t segs,
                                                uint32_t err) {
    const unsigned jm = __match_any_sync(active, k);
    const uint32_t we = __reduce_add_sync(jm, emitted);
    const uint32_t ws = __reduce_add_sync(jm, segs);
    const uint32_t wr = __reduce_or_sync(jm, err);
    if ((threadIdx.x & 31) == (__ffs(jm) - 1)) {
        if (we) atomicAdd(&st->emitted_frame, we);
        if (ws) atomicAdd(&st->segments_frame, ws);
        if (wr) atomicOr(&st->err, wr);
    }
}

// fused photon pass: one thread per photon slot, generate + trace + store + hash insert
template <bool COUNT, bool TEX>
__global__ void __launch_bounds__(128) k_photon(LaunchSet ls) {
    const uint32_t g = grid_tid();
    if (g >= ls.total) return;
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    JobState* st = J.state;
    const uint32_t sidx = g - ls.prefix[k];
    uint32_t err = 0;
    float4 rndv = J.ph.rng[sidx];
    const PhotonRay R = photon_generate<TEX>(J, sidx, st->frame, rndv, err);
    uint32_t slot = 0xFFFFFFFFu;
    TraversalCount tc;
    if (R.cont) {
        const Hit h = trace_exact<true, COUNT>(J.scene, R.org, R.dir, false, err, &tc);
        slot = photon_store(J, st, sidx, h, R.dir, R.flux, R.depth);
    } else {
        photon_terminate(J, sidx);
    }
    J.ph.rng[sidx] = rndv;
    const unsigned active = __activemask();
    hash_insert(J, k, sidx, slot, active);
    photon_counters(st, k, active, R.emitted, R.cont ? 1u : 0u, err);
    if (COUNT) {
        const unsigned jm = __match_any_sync(active, k);
        const uint32_t wn = __reduce_add_sync(jm, tc.nodes);
        const uint32_t wt = __reduce_add_sync(jm, tc.tris);
        const uint32_t ws = __reduce_add_sync(jm, R.cont ? 1u : 0u);
        if ((threadIdx.x & 31) == (__ffs(jm) - 1)) {
            atomicAdd(&st->count_nodes, (unsigned long long)wn);
            atomicAdd(&st->count_tris, (unsigned long long)wt);
            atomicAdd(&st->count_segments, (unsigned long long)ws);
        }
    }
}

// ----------------------------------------------------------------------------------------------
// wavefront photon pass: generate -> trace (persistent, dynamic ray fetch) -> store
// ----------------------------------------------------------------------------------------------
// generate: emit/bounce every slot; RR-terminated photons are finished here, the others append
// their ray to the queue (warp-aggregated append)
//
// The block's slots are first reordered so that the emissions (a photon with no previous hit or
// at the bounce limit) come before the bounces: each warp then runs one of the two paths (the
// state written is per slot, so the order of work changes nothing).
template <bool TEX>
__global__ void __launch_bounds__(128) k_photon_gen(LaunchSet ls, RayQueue q) {
    // the slot and its record in processing order (the loads of every slot's record are issued
    // together, before the reorder)
    __shared__ uint32_t order[128];
    __shared__ int2 rec_hit[128];
    __shared__ float4 rec_pos[128], rec_flux[128], rec_dir[128], rec_rng[128];
    __shared__ uint32_t warp_emit[4], warp_valid[4];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    {
        const uint32_t g0 = ls.first + grid_tid();
        const bool valid = g0 < ls.total;
        bool emit = false;
        int2 h = make_int2(-1, 0);
        float4 pp, pf, pd, rn;
        if (valid) {
            const int k0 = find_job(ls, g0);
            const JobDesc& J0 = ls.jobs[ls.job_ids[k0]];
            const JobState* st0 = J0.state;
            const uint32_t s0 = g0 - ls.prefix[k0];
            if (st0->frame != 0) h = J0.ph.hit[s0];
            pp = J0.ph.pos[s0];
            pf = J0.ph.flux[s0];
            pd = J0.ph.dir[s0];
            rn = J0.ph.rng[s0];
            emit = h.x < 0 || xadd((float)h.y, 1.0f) >= (float)J0.max_path;
        }
        const unsigned em = __ballot_sync(0xFFFFFFFFu, emit), vm = __ballot_sync(0xFFFFFFFFu, valid);
        if (lane == 0) {
            warp_emit[warp] = __popc(em);
            warp_valid[warp] = __popc(vm);
        }
        __syncthreads();
        uint32_t e_before = 0, v_before = 0, e_total = 0;
        for (uint32_t w = 0; w < 4; w++) {
            if (w < warp) {
                e_before += warp_emit[w];
                v_before += warp_valid[w];
            }
            e_total += warp_emit[w];
        }
        const unsigned below = (1u << lane) - 1u;
        if (valid) {
            // emissions at [0, e_total), bounces after them
            const uint32_t dst = emit ? e_before + __popc(em & below)
                                      : e_total + (v_before - e_before) + __popc(vm & ~em & below);
            order[dst] = g0;
            rec_hit[dst] = h;
            rec_pos[dst] = pp;
            rec_flux[dst] = pf;
            rec_dir[dst] = pd;
            rec_rng[dst] = rn;
        }
        __syncthreads();
        if (threadIdx.x >= warp_valid[0] + warp_valid[1] + warp_valid[2] + warp_valid[3]) return;
    }
    const uint32_t g = order[threadIdx.x];
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    JobState* st = J.state;
    const uint32_t sidx = g - ls.prefix[k];
    uint32_t err = 0;
    const uint32_t t = threadIdx.x;
    float4 rndv = rec_rng[t];
    const PhotonRay R = photon_generate<TEX>(J, rec_hit[t], rec_pos[t], rec_flux[t], rec_dir[t], rndv, err);
    J.ph.rng[sidx] = rndv;
    if (R.cont) {
        J.ph.flux[sidx] = f4(R.flux, 0.0f);  // flux before the segment, read back by k_photon_store
        J.ph.hit[sidx] = make_int2(-1, (int)R.depth);
    } else {
        photon_terminate(J, sidx);
    }
    const unsigned active = __activemask();
    const unsigned live = __ballot_sync(active, R.cont);
    uint32_t base = 0;
    const int leader = __ffs(active) - 1;
    if ((int)(threadIdx.x & 31) == leader && live) base = atomicAdd(&q.counters[0], __popc(live));
    base = __shfl_sync(active, base, leader);
    if (R.cont) {
        const uint32_t qi = base + __popc(live & ((1u << (threadIdx.x & 31)) - 1));
        q.org[qi] = make_float4(R.org.x, R.org.y, R.org.z, __uint_as_float(g));
        q.dir[qi] = make_float4(R.dir.x, R.dir.y, R.dir.z, 0.0f);
        if (q.key) {
            // lanes with the same bin take consecutive ranks from one atomic
            const uint32_t bin = q.bin_rank[ray_bin(J.scene, R.org, R.dir)];
            const unsigned same = __match_any_sync(live, bin);
            const int lead = __ffs(same) - 1;
            uint32_t rb = 0;
            if ((int)(threadIdx.x & 31) == lead) rb = atomicAdd(&q.bins[bin], __popc(same));
            rb = __shfl_sync(same, rb, lead);
            q.key[qi] = make_uint2(bin, rb + __popc(same & ((1u << (threadIdx.x & 31)) - 1)));
        }
    }
    photon_counters(st, k, active, R.emitted, R.cont ? 1u : 0u, err);
}

// exclusive scan of the bin counts in place (one block of 1024 threads, 96 bins per thread)
__global__ void __launch_bounds__(1024) k_ray_bins_scan(uint32_t* bins) {
    constexpr uint32_t kPer = kRayBins / 1024;
    static_assert(kRayBins % 1024 == 0 && kPer % 4 == 0, "bin count must split into uint4 chunks");
    __shared__ uint32_t warp_sums[32];
    uint4* v = reinterpret_cast<uint4*>(bins) + threadIdx.x * (kPer / 4);
    uint32_t sum = 0;
#pragma unroll 4
    for (uint32_t i = 0; i < kPer / 4; i++) {
        const uint4 x = v[i];
        sum += x.x + x.y + x.z + x.w;
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if ((int)lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane], wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if ((int)lane >= o) wi += y;
        }
        warp_sums[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = warp_sums[warp] + incl - sum;
#pragma unroll 4
    for (uint32_t i = 0; i < kPer / 4; i++) {
        uint4 x = v[i];
        const uint32_t a = x.x, b = x.y, c = x.z, d = x.w;
        x.x = run;
        x.y = run + a;
        x.z = run + a + b;
        x.w = run + a + b + c;
        run += a + b + c + d;
        v[i] = x;
    }
}

// the bins' traversal order, from the mean walk of their rays since the last reorder (at most once
// per 8 frames; the frame kernel counts them): the longest first, so that the persistent traversal
// starts its longest walks early and its drain (lanes idle while the last walks finish) is short
// -- a longest-processing-time-first schedule.  One
// block: the means quantised to 256 keys (0: no ray since the last reorder, placed last); a
// stable counting sort by descending key, rounds of 1024 bins in bin order, each lane's place
// among equal keys from the warp histograms of the round.  Any order gives the same results (the
// rays are independent); this one is deterministic.
__global__ void __launch_bounds__(1024) k_ray_bins_order(RayQueue q) {
    constexpr uint32_t kKeys = 256, kRounds = kRayBins / 1024;
    static_assert(kRayBins % 1024 == 0, "bins must split into rounds of 1024");
    __shared__ uint32_t base[kKeys], cursor[kKeys];
    __shared__ uint32_t hist[32][kKeys];  // [warp][key]: counts of the round, then offsets
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // at most once per 8 frames (with an eye pass every frame the sort would cost a few percent)
    if (q.counters[7] < 8u) return;
    if (t < kKeys) {
        base[t] = 0;
        cursor[t] = 0;
    }
    __syncthreads();
    if (t == 0) q.counters[7] = 0;
    uint32_t key[kRounds];
#pragma unroll
    for (uint32_t r = 0; r < kRounds; r++) {
        const unsigned long long c = q.bin_cost[q.bin_rank[r * 1024 + t]];
        const uint32_t n = (uint32_t)c, mean = n ? (uint32_t)(c >> 32) / n : 0u;
        const uint32_t k = n ? 1u + min(254u, mean < 128u ? mean : 128u + (mean - 128u) / 8u) : 0u;
        key[r] = kKeys - 1u - k;  // descending mean
        atomicAdd(&base[key[r]], 1u);
    }
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the key totals, 8 keys per lane
        uint32_t v[kKeys / 32], s = 0;
#pragma unroll
        for (uint32_t i = 0; i < kKeys / 32; i++) {
            v[i] = base[lane * (kKeys / 32) + i];
            s += v[i];
        }
        uint32_t incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if ((int)lane >= o) incl += y;
        }
        uint32_t run = incl - s;
#pragma unroll
        for (uint32_t i = 0; i < kKeys / 32; i++) {
            base[lane * (kKeys / 32) + i] = run;
            run += v[i];
        }
    }
    for (uint32_t i = t; i < kRayBins; i += 1024) q.bin_cost[i] = 0ull;  // every cost was read above
    uint32_t rank[kRounds];
#pragma unroll
    for (uint32_t r = 0; r < kRounds; r++) {
        for (uint32_t i = t; i < 32 * kKeys; i += 1024) (&hist[0][0])[i] = 0u;
        __syncthreads();
        const uint32_t k = key[r];
        const unsigned same = __match_any_sync(0xFFFFFFFFu, k);
        if ((int)lane == __ffs(same) - 1) hist[warp][k] = __popc(same);
        __syncthreads();
        if (t < kKeys) {  // offsets of each warp's lanes among the key's bins so far
            uint32_t run = cursor[t];
            for (uint32_t w = 0; w < 32; w++) {
                const uint32_t c = hist[w][t];
                hist[w][t] = run;
                run += c;
            }
            cursor[t] = run;
        }
        __syncthreads();
        rank[r] = base[k] + hist[warp][k] + __popc(same & ((1u << lane) - 1u));
        __syncthreads();
    }
#pragma unroll
    for (uint32_t r = 0; r < kRounds; r++) q.bin_rank[r * 1024 + t] = rank[r];
}

// perm[offset of the bin + rank] = queue index
__global__ void __launch_bounds__(256) k_ray_bins_scatter(RayQueue q) {
    const uint32_t qi = grid_tid();
    if (qi >= q.counters[0]) return;
    const uint2 kr = q.key[qi];
    q.perm[q.bins[kr.x] + kr.y] = qi;
}

// trace: persistent warps; a lane whose ray finished fetches the next one from the queue, so
// lanes stay busy while their neighbours walk longer paths (dynamic fetch)
template <bool COUNT>
__global__ void __launch_bounds__(128, 9) k_trace_photons(LaunchSet ls, RayQueue q) {
    const uint32_t total = q.counters[0];
    const int refill = q.refill_steps ? (int)q.refill_steps : 32;
    const unsigned lane = threadIdx.x & 31;
    const uint32_t kNeed = 0xFFFFFFFFu, kDone = 0xFFFFFFFEu;
    uint32_t idx = kNeed;
    const NodeX* nodes = nullptr;
    const float4* tri_isect = nullptr;
    int32_t nn = 0;
    f3 org = mk(0, 0, 0), dir = mk(0, 0, 0), rcp = mk(0, 0, 0), t0 = mk(0, 0, 0);
    Hit h;
    int32_t node = 0, steps = 0;
    uint32_t err = 0;
    int job_k = 0;
    // traversal counters: summed per lane, added to the job's totals when the lane moves to
    // another job's rays and at the end (three 64-bit atomics per ray would serialise the kernel)
    TraversalCount tc;
    uint32_t tc_segs = 0;
    int tc_job = -1;
    auto flush_counts = [&]() {
        if (tc_job >= 0 && tc_segs) {
            JobState* st = ls.jobs[ls.job_ids[tc_job]].state;
            atomicAdd(&st->count_nodes, (unsigned long long)tc.nodes);
            atomicAdd(&st->count_tris, (unsigned long long)tc.tris);
            atomicAdd(&st->count_segments, (unsigned long long)tc_segs);
        }
        tc.nodes = tc.tris = 0;
        tc_segs = 0;
    };
    for (;;) {
        const bool need = idx == kNeed;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(&q.counters[1], __popc(m));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (need) {
                idx = base + __popc(m & ((1u << lane) - 1));
                if (idx >= total) {
                    idx = kDone;
                } else {
                    if (q.perm) idx = q.perm[idx];
                    const float4 o = q.org[idx], d = q.dir[idx];
                    const uint32_t g = __float_as_uint(o.w);
                    const int nk = find_job(ls, g);
                    if (err && nk != job_k) {  // an error belongs to the job whose ray raised it
                        atomicOr(&ls.jobs[ls.job_ids[job_k]].state->err, err);
                        err = 0;
                    }
                    job_k = nk;
                    if (COUNT && job_k != tc_job) {
                        flush_counts();
                        tc_job = job_k;
                    }
                    const DevScene& S = ls.jobs[ls.job_ids[job_k]].scene;
                    org = mk(o.x, o.y, o.z);
                    dir = mk(d.x, d.y, d.z);
                    nn = (int32_t)S.num_nodes;
                    nodes = S.nodes + (size_t)cube_face(dir) * nn;
                    tri_isect = S.tri_isect;
                    rcp = mk(xdiv(1.0f, dir.x), xdiv(1.0f, dir.y), xdiv(1.0f, dir.z));
                    t0 = mul(neg(rcp), org);
                    h.t = 1.0e30f;
                    h.tri = -1;
                    h.mat = -1;
                    h.bu = h.bv = h.bw = 0.0f;
                    node = 0;
                    steps = 0;
                    if (slab_degenerate(dir)) {
                        // walks most of the tree: left to k_trace_photons_coop
                        q.slow[atomicAdd(&q.counters[2], 1u)] = idx;
                        idx = kNeed;
                    }
                }
            }
        }
        if (__all_sync(0xFFFFFFFFu, idx == kDone)) break;
        // the tail: once the queue is drained, a warp left with a few long walks hands them to
        // k_trace_photons_tail, which finishes each with all 32 lanes of a warp, resumed where the
        // lane stands (coop_trace_exact_from, the same result bit for bit): a walk's chain of
        // dependent node loads becomes windows of 32 loads in flight
        if (q.tail_lanes) {
            const unsigned act = __ballot_sync(0xFFFFFFFFu, idx < kDone);
            const unsigned drained = __ballot_sync(0xFFFFFFFFu, idx == kDone);
            if (drained && act && (uint32_t)__popc(act) <= q.tail_lanes) {
                if (idx < kDone) {
                    q.hit[idx] = make_float4(__int_as_float(h.tri), h.bu, h.bv, h.bw);
                    q.tail_state[idx] = make_float4(h.t, __int_as_float(h.mat), __int_as_float(node),
                                                    __int_as_float(steps));
                    q.tail_list[atomicAdd(&q.counters[4], 1u)] = idx;
                    idx = kDone;
                }
                continue;  // every walk of the warp is handed over; the next iteration leaves the loop
            }
        }
        if (idx >= kDone) continue;
        bool finished = false;
#pragma unroll 1
        for (int it = 0; it < refill; it++) {
            if (steps++ > nn) {
                err |= kErrWatchdogTraverse;
                finished = true;
                break;
            }
            float4 A, B;
            ldg32(nodes + node, A, B);
            if (COUNT) tc.nodes++;
            const float lx = xadd(xmul(rcp.x, A.x), t0.x), ly = xadd(xmul(rcp.y, A.y), t0.y), lz = xadd(xmul(rcp.z, A.z), t0.z);
            const float hx = xadd(xmul(rcp.x, B.x), t0.x), hy = xadd(xmul(rcp.y, B.y), t0.y), hz = xadd(xmul(rcp.z, B.z), t0.z);
            const float tmin = fmax3(fminf(lx, hx), fminf(ly, hy), fminf(lz, hz));
            const float tmax = fmin3(fmaxf(lx, hx), fmaxf(ly, hy), fmaxf(lz, hz));
            const bool hit = (tmin <= tmax) && (tmin <= h.t) && (tmax >= 0.0f);
            const int32_t tri = __float_as_int(B.w);
            if (hit && tri >= 0 && !(tri & kEmitterBit)) {
                if (COUNT) tc.tris++;
                const float4 a = __ldg(&tri_isect[(size_t)tri * 3 + 0]);
                const float4 b = __ldg(&tri_isect[(size_t)tri * 3 + 1]);
                const float4 c = __ldg(&tri_isect[(size_t)tri * 3 + 2]);
                const f3 v0 = mk(a.x, a.y, a.z), e0 = mk(a.w, b.x, b.y), e1 = mk(b.z, b.w, c.x);
                const f3 pv = cross(dir, e1);
                const float det = dot(e0, pv);
                const f3 tv = sub(org, v0);
                const f3 qv = cross(tv, e0);
                const float u = xdiv(dot(tv, pv), det);
                const float v = xdiv(dot(dir, qv), det);
                const float tt = xdiv(dot(e1, qv), det);
                const float w = xsub(xsub(1.0f, u), v);
                if (u >= 0.0f && v >= 0.0f && tt >= 0.0f && w >= 0.0f && tt < h.t) {
                    h.t = tt;
                    h.tri = tri;
                    h.mat = __float_as_int(c.y);
                    h.bu = v;
                    h.bv = w;
                    h.bw = u;
                }
            }
            const int32_t next = hit ? node + 1 : __float_as_int(A.w);
            if (next < 0 || next >= nn) {
                finished = true;
                break;
            }
            node = next;
        }
        if (finished) {
            q.hit[idx] = make_float4(__int_as_float(h.tri), h.bu, h.bv, h.bw);
            if (q.perm) bin_cost_add(q, q.key[idx].x, (uint32_t)steps);
            if (COUNT) tc_segs++;
            idx = kNeed;
        }
    }
    if (COUNT) flush_counts();
    if (err) atomicOr(&ls.jobs[ls.job_ids[job_k]].state->err, err);
}

// the walks k_trace_photons handed over once its queue was drained: one warp per walk, resumed at
// the node, closest hit and step count where its lane stopped
template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace_photons_tail(LaunchSet ls, RayQueue q) {
    const uint32_t n = q.counters[4];
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    const unsigned lane = threadIdx.x & 31;
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n; w += warps) {
        const uint32_t idx = q.tail_list[w];
        const float4 o = q.org[idx], d = q.dir[idx], hr = q.hit[idx], ts = q.tail_state[idx];
        const int job_k = find_job(ls, __float_as_uint(o.w));
        const JobDesc& J = ls.jobs[ls.job_ids[job_k]];
        Hit h0;
        h0.t = ts.x;
        h0.mat = __float_as_int(ts.y);
        h0.tri = __float_as_int(hr.x);
        h0.bu = hr.y;
        h0.bv = hr.z;
        h0.bw = hr.w;
        uint32_t err = 0;
        TraversalCount ct;
        const Hit h = coop_trace_exact_from<true, COUNT>(J.scene, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), false, err,
                                                         &ct, __float_as_int(ts.z), h0, (uint32_t)__float_as_int(ts.w));
        if (lane == 0) {
            q.hit[idx] = make_float4(__int_as_float(h.tri), h.bu, h.bv, h.bw);
            if (err) atomicOr(&J.state->err, err);
            if (COUNT) {
                atomicAdd(&J.state->count_nodes, (unsigned long long)ct.nodes);
                atomicAdd(&J.state->count_tris, (unsigned long long)ct.tris);
                atomicAdd(&J.state->count_segments, 1ull);
            }
        }
    }
}

// the rays k_trace_photons set aside (slab_degenerate directions), one block of 1024 threads per
// ray (block_trace_exact)
template <bool COUNT>
__global__ void __launch_bounds__(kBlockWalk) k_trace_photons_coop(LaunchSet ls, RayQueue q) {
    __shared__ BlockWalkShared sh;
    const uint32_t n = q.counters[2];
    for (uint32_t w = blockIdx.x; w < n; w += gridDim.x) {
        const uint32_t idx = q.slow[w];
        const float4 o = q.org[idx], d = q.dir[idx];
        const int job_k = find_job(ls, __float_as_uint(o.w));
        const JobDesc& J = ls.jobs[ls.job_ids[job_k]];
        uint32_t err = 0;
        TraversalCount ct;
        const Hit h = block_trace_exact<true, COUNT>(J.scene, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), false, err, &ct,
                                                     sh);
        if (threadIdx.x == 0) {
            q.hit[idx] = make_float4(__int_as_float(h.tri), h.bu, h.bv, h.bw);
            atomicAdd(&J.state->coop_segments, 1ull);
            if (err) atomicOr(&J.state->err, err);
            if (COUNT) {
                atomicAdd(&J.state->count_nodes, (unsigned long long)ct.nodes);
                atomicAdd(&J.state->count_tris, (unsigned long long)ct.tris);
                atomicAdd(&J.state->count_segments, 1ull);
            }
        }
    }
}

// store: shade the hit of each queued ray, write the photon record, insert it into the grid
__global__ void __launch_bounds__(128) k_photon_store(LaunchSet ls, RayQueue q, uint32_t grid_shift) {
    const uint32_t qi = grid_tid();
    if (qi >= q.counters[0]) return;
    const float4 o = q.org[qi], d = q.dir[qi], hr = q.hit[qi];
    const uint32_t g = __float_as_uint(o.w);
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    const JobState* st = J.state;
    const uint32_t sidx = g - ls.prefix[k];
    Hit h;
    h.tri = __float_as_int(hr.x);
    h.bu = hr.y;
    h.bv = hr.z;
    h.bw = hr.w;
    h.mat = h.tri >= 0 ? __float_as_int(__ldg(&J.scene.tri_isect[(size_t)h.tri * 3 + 2]).y) : -1;
    const float4 f = J.ph.flux[sidx];
    const int depth = J.ph.hit[sidx].y;
    const uint32_t slot = photon_store(J, st, sidx, h, mk(d.x, d.y, d.z), mk(f.x, f.y, f.z), (float)depth, grid_shift);
    q.hit[qi].x = __uint_as_float(slot);  // for the slot records of the mixed path
    hash_insert(J, k, sidx, slot, __activemask());
}

// ----------------------------------------------------------------------------------------------
// k_gather: progressive.fs (:98-142, AccumulatePhotons :65-95)
// ----------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_gather(LaunchSet ls) {
    const uint32_t g = grid_tid();
    if (g >= ls.total) return;
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    JobState* st = J.state;
    const uint32_t p = g - ls.prefix[k];
    const uint32_t frame = st->frame;
    if (p == 0) {
        // NumPhotons += int(sum) (glslppm.cpp:397) once the photon pass of this frame is done
        const uint32_t e = st->emitted_frame;
        st->num_photons_f32 = xadd(st->num_photons_f32, (float)(int)e);
        st->num_photons += e;
        st->photon_segments += st->segments_frame;
    }
    float4 qfr = frame == 0 ? make_float4(0.0f, 0.0f, 0.0f, st->r0) : J.px.flux_r[p];
    float4 qe = J.px.emi_n[p];
    if (J.px.tri[p] >= 0) {
        const float G = st->grid_scale;
        const float hs1 = st->hash_scale1;
        const float hn = (float)J.hash_num;
        const float alpha = J.alpha;
        const f3 bbmin = mk(st->bbmin[0], st->bbmin[1], st->bbmin[2]);
        const f3 qp = xyz(J.px.pos[p]), qn = xyz(J.px.nrm[p]), qr = xyz(J.px.refl[p]);
        float N = qe.w, R = qfr.w;
        f3 tau = xyz(qfr);
        const f3 ii = mk(floorf(xsub(xmul(fabsf(xsub(qp.x, bbmin.x)), G), 0.5f)),
                         floorf(xsub(xmul(fabsf(xsub(qp.y, bbmin.y)), G), 0.5f)),
                         floorf(xsub(xmul(fabsf(xsub(qp.z, bbmin.z)), G), 0.5f)));
        f3 flux = mk(0, 0, 0);
        float M = 0.0f;
        // the eight cells' slots and winners first (independent loads in flight together), then
        // the candidate photons' positions, then the accumulation in cell order (the sum's order
        // is progressive.fs's)
        uint32_t slot[8], win[8];
        hash_cells8(ii, G, hs1, hn, slot);
        const uint32_t clipped_only = J.PW * J.PH;  // every photon of the slot clipped: photon 0
#pragma unroll
        for (int c = 0; c < 8; c++) {
            win[c] = __ldg(&J.winner[slot[c]]);
            if (win[c] == clipped_only) win[c] = 0u;
        }
        uint32_t inside = 0;
        // the cells' bounds from the table k_cell_bounds made for this grid (the same values as
        // the division below), when the 2x2x2 block lies inside it
        const float tn = (float)st->cell_table_n;
        const bool table = J.cell_bounds && ii.x >= 0.0f && ii.y >= 0.0f && ii.z >= 0.0f && ii.x + 2.0f < tn &&
                           ii.y + 2.0f < tn && ii.z + 2.0f < tn;
        const uint32_t tx = table ? (uint32_t)ii.x : 0u, ty = table ? (uint32_t)ii.y : 0u,
                       tz = table ? (uint32_t)ii.z : 0u;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            if (win[c] == kEmptySlot) continue;  // the cleared texel: photon 0 weighted by count 0
            const f3 cell = mk(xadd(ii.x, (float)(c & 1)), xadd(ii.y, (float)((c >> 1) & 1)), xadd(ii.z, (float)(c >> 2)));
            const float4 pp = __ldg(&J.ph.pos[win[c]]);
            f3 rmin, rmax;
            if (table) {
                const float* T = J.cell_bounds;
                const uint32_t cx = tx + (c & 1), cy = ty + ((c >> 1) & 1), cz = tz + (c >> 2);
                rmin = mk(__ldg(&T[cx]), __ldg(&T[kCellTable + cy]), __ldg(&T[2 * kCellTable + cz]));
                rmax = mk(__ldg(&T[cx + 1]), __ldg(&T[kCellTable + cy + 1]), __ldg(&T[2 * kCellTable + cz + 1]));
            } else {
                rmin = mk(xadd(xdiv(cell.x, G), bbmin.x), xadd(xdiv(cell.y, G), bbmin.y), xadd(xdiv(cell.z, G), bbmin.z));
                rmax = mk(xadd(xdiv(xadd(cell.x, 1.0f), G), bbmin.x), xadd(xdiv(xadd(cell.y, 1.0f), G), bbmin.y),
                          xadd(xdiv(xadd(cell.z, 1.0f), G), bbmin.z));
            }
            if (pp.x > rmin.x && pp.y > rmin.y && pp.z > rmin.z && pp.x < rmax.x && pp.y < rmax.y && pp.z < rmax.z &&
                length(sub(xyz(pp), qp)) < R)
                inside |= 1u << c;
        }
#pragma unroll
        for (int c = 0; c < 8; c++) {
            if (!((inside >> c) & 1u)) continue;
            const float4 pd = __ldg(&J.ph.dir[win[c]]);
            if (dot(qn, neg(xyz(pd))) > 0.0f) {
                const float4 pf = __ldg(&J.ph.flux[win[c]]);
                const float cnt = (float)__ldg(&J.count[slot[c]]);
                flux = add(flux, scl(xyz(pf), cnt));
                M = xadd(M, cnt);
            }
        }
        flux = mul(flux, scl(qr, 3.183099627e-01f));
        const float gg = fminf(xdiv(xadd(N, xmul(alpha, M)), xadd(N, M)), 1.0f);
        R = xmul(R, xsqrt(gg));
        N = xadd(N, xmul(M, alpha));
        tau = scl(add(tau, flux), gg);
        qfr = f4(tau, R);
        qe.w = N;
        J.px.emi_n[p] = qe;
    }
    J.px.flux_r[p] = qfr;
}

// ----------------------------------------------------------------------------------------------
// k_resolve: re.fs
// ----------------------------------------------------------------------------------------------
__global__ void k_resolve(LaunchSet ls, uint32_t display) {
    const uint32_t g = grid_tid();
    if (g >= ls.total) return;
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    const uint32_t p = g - ls.prefix[k];
    const float4 fr = J.px.flux_r[p];
    const float4 qe = J.px.emi_n[p];
    const float total = J.state->num_photons_f32;
    const float den = xmul(xmul(xmul(fr.w, fr.w), 3.141592f), total);
    float L[3] = {xadd(xdiv(fr.x, den), qe.x), xadd(xdiv(fr.y, den), qe.y), xadd(xdiv(fr.z, den), qe.z)};
    for (int c = 0; c < 3; c++) {
        float v = L[c];
        if (display) {
            v = xsub(1.0f, sppm_fexp(xmul(-v, 60000.0f)));
            if (v < 0.0031308f) v = xmul(12.92f, v);
            else v = xsub(xmul(xadd(1.0f, 0.055f), sppm_fpow(v, 0.416666666667f)), 0.055f);
        }
        J.image[(size_t)p * 3 + c] = v;
    }
}

// ----------------------------------------------------------------------------------------------
// stage-level hash build on caller arrays (sppm_hash_build)
// ----------------------------------------------------------------------------------------------
__global__ void k_hash_clear(uint32_t* winner, uint32_t* count, uint32_t n) {
    const uint32_t g = grid_tid();
    if (g < n) {
        winner[g] = kEmptySlot;
        count[g] = 0;
    }
}

__global__ void k_hash_build(const float4* pos, const float4* flux, uint32_t pw, uint32_t ph, uint32_t hash_num,
                             float bx, float by, float bz, float G, uint32_t flags, uint32_t* winner, uint32_t* count) {
    const uint32_t id = grid_tid();
    if (id >= pw * ph) return;
    const float hs1 = xdiv(4194304.0f, G);
    const float4 f = flux[id];
    const bool store = !(f.x < 0.0f);
    uint32_t slot = 0;
    if (store) {
        const float4 pp = pos[id];
        const f3 cell = mk(floorf(xmul(xsub(pp.x, bx), G)), floorf(xmul(xsub(pp.y, by), G)), floorf(xmul(xsub(pp.z, bz), G)));
        slot = hash_cell(cell, G, hs1, (float)hash_num);
    }
    const bool clipped = (flags & SPPM_FLAG_GL_DEPTH_CLIP) && id >= (ph - 1) * pw + (pw + 1) / 2;
    const unsigned peers = __match_any_sync(__activemask(), store ? slot : 0xFFFFFFFFu);
    if (store) {
        const uint32_t n = __popc(peers);
        const uint32_t wmin = __reduce_min_sync(peers, clipped ? 0xFFFFFFFFu : id);
        if ((threadIdx.x & 31) == (__ffs(peers) - 1)) {
            atomicAdd(&count[slot], n);
            if (wmin != 0xFFFFFFFFu) atomicMin(&winner[slot], wmin);
        }
    }
}

// pinned math on the device, for the accuracy / determinism tests
__global__ void k_fpmath(int fn, const float* x, const float* y, float* out, uint32_t n) {
    const uint32_t i = grid_tid();
    if (i >= n) return;
    float r;
    switch (fn) {
        case 0: r = sppm_fsin(x[i]); break;
        case 1: r = sppm_fcos(x[i]); break;
        case 2: r = sppm_fpow(x[i], y[i]); break;
        case 3: r = sppm_fexp(x[i]); break;
        case 4: r = sppm_flog2(x[i]); break;
        default: r = sppm_fexp2(x[i]); break;
    }
    out[i] = r;
}

// single rays through the exact traversal: mode 0 one thread per ray (trace_exact), mode 1 one
// warp per ray (coop_trace_exact), mode 2 one block per ray (block_trace_exact), mode 3 the mixed
// path's 4-wide quantised traversal one per thread (trace4); photon rays skip emitters, eye rays
// may cull back faces
template <bool PHOTON>
__global__ void __launch_bounds__(1024) k_debug_trace(DevScene s, const float* org, const float* dir, uint32_t n,
                                                     int cull, int mode, int32_t* tri, float* t, uint32_t* err) {
    uint32_t e = 0;
    if (mode == 2) {
        __shared__ BlockWalkShared sh;
        for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
            TraversalCount ct;
            const Hit h = block_trace_exact<PHOTON, false>(s, mk(org[3 * i], org[3 * i + 1], org[3 * i + 2]),
                                                           mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]), cull != 0, e,
                                                           &ct, sh);
            if (threadIdx.x == 0) {
                tri[i] = h.tri;
                t[i] = h.t;
            }
        }
    } else if (mode == 0) {
        const uint32_t i = grid_tid();
        if (i >= n) return;
        const Hit h = trace_exact<PHOTON>(s, mk(org[3 * i], org[3 * i + 1], org[3 * i + 2]),
                                          mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]), cull != 0, e);
        tri[i] = h.tri;
        t[i] = h.t;
    } else if (mode == 3) {
        // the mixed path's 4-wide quantised traversal (the eye pass's trace4)
        const uint32_t i = grid_tid();
        if (i >= n) return;
        const f3 d3 = mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
        const Hit4 h = trace4<PHOTON>(s.nodes4, s.tri_isect, mk(org[3 * i], org[3 * i + 1], org[3 * i + 2]), d3,
                                      cull != 0, PHOTON ? 1.0e30f : 1.0e20f, e,
                                      s.tri_rank ? s.tri_rank + (size_t)cube_face(d3) * s.num_tris : nullptr);
        tri[i] = h.tri;
        t[i] = h.t;
    } else {
        const uint32_t warps = gridDim.x * (blockDim.x >> 5);
        for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
            TraversalCount ct;
            const Hit h = coop_trace_exact<PHOTON, false>(s, mk(org[3 * i], org[3 * i + 1], org[3 * i + 2]),
                                                          mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]), cull != 0,
                                                          e, &ct);
            if ((threadIdx.x & 31) == 0) {
                tri[i] = h.tri;
                t[i] = h.t;
            }
        }
    }
    if (e) atomicOr(err, e);
}

__global__ void k_copy_from_host(unsigned long long* dst, const unsigned long long* src, uint32_t words) {
    for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
}

__global__ void k_copy_descs(DescCopy list) {
    static_assert(sizeof(JobDesc) % 8 == 0, "JobDesc is copied in 8-byte words");
    if (blockIdx.x >= list.n) return;
    auto* dst = reinterpret_cast<unsigned long long*>(list.dst[blockIdx.x]);
    const auto* src = reinterpret_cast<const unsigned long long*>(list.src[blockIdx.x]);
    for (uint32_t w = threadIdx.x; w < sizeof(JobDesc) / 8; w += blockDim.x) dst[w] = src[w];
}

// one block per listed job: its JobState word by word
__global__ void k_gather_states(const JobDesc* jobs, StateGather list, JobState* out) {
    static_assert(sizeof(JobState) % 4 == 0, "JobState is copied in 32-bit words");
    if (blockIdx.x >= list.n) return;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs[list.slot[blockIdx.x]].state);
    uint32_t* dst = reinterpret_cast<uint32_t*>(out + blockIdx.x);
    for (uint32_t w = threadIdx.x; w < sizeof(JobState) / 4; w += blockDim.x) dst[w] = src[w];
}

// ----------------------------------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------------------------------
static inline uint32_t blocks_for(uint32_t n, uint32_t b) { return (n + b - 1) / b; }

void launch_copy_from_host(void* dst, const void* src_mapped, size_t bytes, cudaStream_t s) {
    k_copy_from_host<<<1, 64, 0, s>>>(static_cast<unsigned long long*>(dst),
                                       static_cast<const unsigned long long*>(src_mapped), (uint32_t)(bytes / 8));
}
void launch_copy_descs(const DescCopy& list, cudaStream_t s) {
    if (list.n) k_copy_descs<<<list.n, 64, 0, s>>>(list);
}
void launch_gather_states(const JobDesc* jobs, const StateGather& list, JobState* out, cudaStream_t s) {
    if (list.n) k_gather_states<<<list.n, 64, 0, s>>>(jobs, list, out);
}
void launch_frame_begin(const LaunchSet& ls, const RayQueue& q, cudaStream_t s) {
    const uint32_t n = q.bins && ls.total < kRayBins ? kRayBins : ls.total;
    if (ls.total) k_frame_begin<<<blocks_for(n, 256), 256, 0, s>>>(ls, q);
}
// block sizes: a multiple of 32 up to the kernel's launch bound (0 or anything else: the bound)
static uint32_t block_or(uint32_t block, uint32_t bound) {
    return block >= 32 && block <= bound && block % 32 == 0 ? block : bound;
}

template <bool TEX>
static void launch_eye_t(const LaunchSet& ls, const RayQueue& q, bool mixed, uint32_t block, cudaStream_t s) {
    const uint32_t b = block_or(block, 128);
    if (mixed) {
        k_eye<true, TEX><<<blocks_for(ls.total, b), b, 0, s>>>(ls, nullptr, nullptr, 0);
        return;
    }
    k_eye<false, TEX><<<blocks_for(ls.total, b), b, 0, s>>>(ls, q.counters + 3, q.eye_deferred, kEyeDeferred);
    // a fixed grid (the count is on the device): blocks beyond the deferred pixels exit at once
    k_eye_coop<TEX><<<32, kBlockWalk, 0, s>>>(ls, q.counters + 3, q.eye_deferred, kEyeDeferred);
}
void launch_eye(const LaunchSet& ls, const RayQueue& q, bool mixed, bool textured, uint32_t block, cudaStream_t s) {
    if (!ls.total) return;
    if (textured) launch_eye_t<true>(ls, q, mixed, block, s);
    else launch_eye_t<false>(ls, q, mixed, block, s);
}
void launch_grid(const JobDesc* jobs, const uint32_t* job_ids, uint32_t njobs, cudaStream_t s) {
    if (njobs) k_grid<<<blocks_for(njobs, 64), 64, 0, s>>>(jobs, job_ids, njobs);
}
void launch_cell_bounds(const JobDesc* jobs, const uint32_t* job_ids, uint32_t njobs, cudaStream_t s) {
    if (njobs) k_cell_bounds<<<njobs, 256, 0, s>>>(jobs, job_ids);
}
void launch_photon_fp32(const LaunchSet& ls, bool count, bool textured, cudaStream_t s) {
    if (!ls.total) return;
    const uint32_t b = blocks_for(ls.total, 128);
    if (count && textured) k_photon<true, true><<<b, 128, 0, s>>>(ls);
    else if (count) k_photon<true, false><<<b, 128, 0, s>>>(ls);
    else if (textured) k_photon<false, true><<<b, 128, 0, s>>>(ls);
    else k_photon<false, false><<<b, 128, 0, s>>>(ls);
}

void launch_photon_gen_fp32(const LaunchSet& ls, const RayQueue& q, bool textured, cudaStream_t s) {
    if (ls.total <= ls.first) return;
    const uint32_t n = ls.total - ls.first;
    if (textured) k_photon_gen<true><<<blocks_for(n, 128), 128, 0, s>>>(ls, q);
    else k_photon_gen<false><<<blocks_for(n, 128), 128, 0, s>>>(ls, q);
}
void launch_queue_reset(const RayQueue& q, cudaStream_t s) {
    if (q.counters) k_queue_reset<<<blocks_for(kRayBins, 256), 256, 0, s>>>(q);
}
void launch_ray_bins_order(const RayQueue& q, cudaStream_t s) {
    if (q.key && q.bin_rank && q.bin_cost) k_ray_bins_order<<<1, 1024, 0, s>>>(q);
}
void launch_ray_bins(const RayQueue& q, cudaStream_t s) {
    if (!q.key || !q.capacity) return;
    k_ray_bins_scan<<<1, 1024, 0, s>>>(q.bins);
    k_ray_bins_scatter<<<blocks_for(q.capacity, 256), 256, 0, s>>>(q);
}

void launch_trace_photons_fp32(const LaunchSet& ls, const RayQueue& q, bool count, uint32_t persistent_blocks,
                               cudaStream_t s) {
    if (!ls.total) return;
    if (count) k_trace_photons<true><<<persistent_blocks, 128, 0, s>>>(ls, q);
    else k_trace_photons<false><<<persistent_blocks, 128, 0, s>>>(ls, q);
    if (q.tail_lanes && q.tail_list) {
        // one warp per handed-over walk: enough warps for every SM
        if (count) k_trace_photons_tail<true><<<persistent_blocks, 128, 0, s>>>(ls, q);
        else k_trace_photons_tail<false><<<persistent_blocks, 128, 0, s>>>(ls, q);
    }
    launch_trace_photons_coop(ls, q, count, s);
}
void launch_trace_photons_coop(const LaunchSet& ls, const RayQueue& q, bool count, cudaStream_t s) {
    if (!ls.total || !q.slow) return;
    if (count) k_trace_photons_coop<true><<<64, kBlockWalk, 0, s>>>(ls, q);
    else k_trace_photons_coop<false><<<64, kBlockWalk, 0, s>>>(ls, q);
}

void launch_photon_store_fp32(const LaunchSet& ls, const RayQueue& q, uint32_t block, uint32_t grid_shift,
                              cudaStream_t s) {
    const uint32_t b = block_or(block, 128);
    if (ls.total) k_photon_store<<<blocks_for(q.capacity, b), b, 0, s>>>(ls, q, grid_shift);
}

uint32_t trace_photons_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace_photons<false>, 128, 0) != cudaSuccess) n = 4;
    return n > 0 ? (uint32_t)n : 1u;
}
void launch_gather_fp32(const LaunchSet& ls, uint32_t block, cudaStream_t s) {
    const uint32_t b = block_or(block, 256);
    if (ls.total) k_gather<<<blocks_for(ls.total, b), b, 0, s>>>(ls);
}
void launch_resolve_fp32(const LaunchSet& ls, uint32_t display, cudaStream_t s) {
    if (ls.total) k_resolve<<<blocks_for(ls.total, 256), 256, 0, s>>>(ls, display);
}
void launch_hash_build(const float4* pos, const float4* flux, uint32_t pw, uint32_t ph, uint32_t hash_num,
                       const float bbmin[3], float G, uint32_t flags, uint32_t* winner, uint32_t* count, cudaStream_t s) {
    k_hash_clear<<<blocks_for(hash_num, 256), 256, 0, s>>>(winner, count, hash_num);
    const uint32_t n = pw * ph;
    if (n) k_hash_build<<<blocks_for(n, 256), 256, 0, s>>>(pos, flux, pw, ph, hash_num, bbmin[0], bbmin[1], bbmin[2], G, flags, winner, count);
}
void launch_fpmath(int fn, const float* x, const float* y, float* out, uint32_t n, cudaStream_t s) {
    if (n) k_fpmath<<<blocks_for(n, 256), 256, 0, s>>>(fn, x, y, out, n);
}

void launch_debug_trace(const DevScene& sc, const float* org, const float* dir, uint32_t n, bool photon, bool cull,
                        int mode, int32_t* tri, float* t, uint32_t* err, cudaStream_t s) {
    if (!n) return;
    const uint32_t threads = mode == 2 ? kBlockWalk : 128;
    const uint32_t blocks =
        (mode == 0 || mode == 3) ? blocks_for(n, 128) : (mode == 1 ? blocks_for(n, 4) : (n < 256 ? n : 256u));
    if (photon) k_debug_trace<true><<<blocks, threads, 0, s>>>(sc, org, dir, n, cull, mode, tri, t, err);
    else k_debug_trace<false><<<blocks, threads, 0, s>>>(sc, org, dir, n, cull, mode, tri, t, err);
}

}  // namespace sppm_dev

// Mixed-precision SPPM kernels (sppm_config.precision = SPPM_PRECISION_MIXED).
//
// What changes against the plain FP32 path, and why:
//  * photon segments are traced through a 4-wide BVH whose child boxes are 8-bit outward-rounded
//    offsets (64-byte nodes: one node fetch tests four boxes), closest-child-first with a stack;
//    the slab distances are fused multiply-adds widened by a bound on their rounding (never
//    culling a box the exact arithmetic enters) and triangles are tested with the plain path's
//    arithmetic, so the reported triangle, t and barycentrics are the exact traversal's (at an
//    equal t the triangle the exact walk meets first, by the leaf ranks of its ordering) -- which
//    also lets the plain FP32 path trace through this BVH (sppm_tuning.wide_bvh);
//  * the photon a hash slot keeps is stored once per slot as a 32-byte record -- cell (int16 x3),
//    position inside the cell (unorm16 x3), flux (FP16 x3, scaled by 1/(light area * pi)),
//    direction (snorm16 x3) and the slot's photon count -- so the gather reads one sector per cell
//    instead of the winner index, three photon arrays and the count; the in-cell test becomes an
//    integer compare;
//  * flux is gathered in FP32 and the per-pixel statistics N, R^2 and tau are kept as double-float
//    pairs (about 48 significant bits from FP32 arithmetic: GB300's FP64 rate is a small fraction
//    of its FP32 rate).
// Emission/bounce (photon generation), photon records and hashing stay the plain FP32 kernels.
#include <cstdint>

#include <cuda_fp16.h>

#include "bvh4_trace.cuh"
#include "device_common.cuh"
#include "kernels.h"
#include "photon_grid.cuh"

namespace sppm_dev {

constexpr int kTraceBlock = 128;
constexpr int kSmemStack = 16;  // top of each thread's stack, in shared memory (16 KB per block)
constexpr int kLocalStack = kStack - kSmemStack;  // deeper entries, in local memory (rarely touched)

// at an equal t: does the exact walk meet triangle a before triangle b?  (the leaf ranks of the
// ray's ordering; looked up only at ties, so the walk keeps no pointer to them)
__device__ __noinline__ bool met_first(const LaunchSet& ls, int job_k, const Ray4& R, int32_t a, int32_t b) {
    const DevScene& S = ls.jobs[ls.job_ids[job_k]].scene;
    if (!S.tri_rank) return false;
    const int32_t* rank = S.tri_rank + (size_t)cube_face(mk(R.dx, R.dy, R.dz)) * S.num_tris;
    return __ldg(&rank[a]) < __ldg(&rank[b]);
}

// photon segments through the 4-wide BVH: persistent warps with dynamic ray fetch (a lane whose
// ray finished takes the next queued ray), one node per lane per step, closest child first, the
// other hit children on a per-thread stack in shared memory
__global__ void __launch_bounds__(kTraceBlock) k_trace_photons4(LaunchSet ls, RayQueue q) {
    __shared__ int32_t s_node[kSmemStack][kTraceBlock];
    __shared__ float s_t[kSmemStack][kTraceBlock];
    int32_t l_node[kLocalStack];
    float l_t[kLocalStack];
    auto push = [&](int sp_, int32_t n, float t) {
        if (sp_ < kSmemStack) {
            s_node[sp_][threadIdx.x] = n;
            s_t[sp_][threadIdx.x] = t;
        } else {
            l_node[sp_ - kSmemStack] = n;
            l_t[sp_ - kSmemStack] = t;
        }
    };
    const uint32_t total = q.counters[0];
    const int refill = q.refill_steps ? (int)q.refill_steps : 8;
    const unsigned lane = threadIdx.x & 31, tid = threadIdx.x;
    const uint32_t kNeed = 0xFFFFFFFFu, kDone = 0xFFFFFFFEu;
    uint32_t idx = kNeed;
    const Node4Dev* nodes = nullptr;
    const float4* tri_isect = nullptr;
    Ray4 R;
    ray4_setup(R, 0.0f, 0.0f, 0.0f, 1.0f, 1.0f, 1.0f);
    float ht = 1.0e30f, hbu = 0, hbv = 0, hbw = 0;
    int32_t htri = -1, cur = 0;
    int sp = 0;
    uint32_t visits = 0, err = 0;
    int job_k = 0;
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
                    const int nk = find_job(ls, __float_as_uint(o.w));
                    if (err && nk != job_k) {  // an error belongs to the job whose ray raised it
                        atomicOr(&ls.jobs[ls.job_ids[job_k]].state->err, err);
                        err = 0;
                    }
                    job_k = nk;
                    const DevScene& S = ls.jobs[ls.job_ids[job_k]].scene;
                    nodes = S.nodes4;
                    tri_isect = S.tri_isect;
                    ray4_setup(R, o.x, o.y, o.z, d.x, d.y, d.z);
                    ht = 1.0e30f;
                    htri = -1;
                    hbu = hbv = hbw = 0.0f;
                    cur = 0;
                    sp = 0;
                    visits = 0;
                }
            }
        }
        if (__all_sync(0xFFFFFFFFu, idx == kDone)) break;
        if (idx == kDone) continue;
        bool finished = false;
#pragma unroll 1
        for (int it = 0; it < refill && !finished; it++) {
            if (++visits > (1u << 22)) {
                err |= kErrWatchdogTraverse;
                finished = true;
                break;
            }
            const float4* np = reinterpret_cast<const float4*>(nodes + cur);
            float4 w0, w1, w2, w3;
            ldg32(np, w0, w1);
            ldg32(np + 2, w2, w3);
            const int cnt = (int)(__float_as_uint(w0.w) >> 24);
            float t[4];
            bool hit[4];
            Slab4 S;
            slab4_setup(S, R, w0, w2, w3);
            const float tcull = ht * kCullMargin;
            child_box<0>(S, tcull, t[0], hit[0]);
            child_box<1>(S, tcull, t[1], hit[1]);
            child_box<2>(S, tcull, t[2], hit[2]);
            child_box<3>(S, tcull, t[3], hit[3]);
            int32_t c[4] = {__float_as_int(w1.x), __float_as_int(w1.y), __float_as_int(w1.z), __float_as_int(w1.w)};
            // leaf children hit: their triangles, in child order (photons pass through emitters);
            // one copy of the test in a loop over the leaves, so a warp runs it as many times as
            // its lane with the most leaves needs
            uint32_t leaves = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                hit[k] = hit[k] && k < cnt;
                if (!hit[k] || c[k] >= 0) continue;
                hit[k] = false;
                if (!(~c[k] & kEmitterBit)) leaves |= 1u << k;
            }
            while (leaves) {
                const int k = __ffs(leaves) - 1;
                leaves &= leaves - 1;
                const int32_t ck = k == 0 ? c[0] : (k == 1 ? c[1] : (k == 2 ? c[2] : c[3]));
                const int32_t code = ~ck;
                const float4 a = __ldg(&tri_isect[(size_t)code * 3 + 0]);
                const float4 b = __ldg(&tri_isect[(size_t)code * 3 + 1]);
                const float4 cc = __ldg(&tri_isect[(size_t)code * 3 + 2]);
                float tt, u, v, w;
                if (tri_hit_exact(a, b, cc, mk(R.ox, R.oy, R.oz), mk(R.dx, R.dy, R.dz), false, tt, u, v, w) &&
                    (tt < ht || (tt == ht && htri >= 0 && met_first(ls, job_k, R, code, htri)))) {
                    ht = tt;
                    htri = code;
                    hbu = v;
                    hbv = w;
                    hbw = u;
                }
            }
            // internal children hit before the current closest hit, sorted near to far
            const float tcull2 = ht * kCullMargin;
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (!(hit[k] && t[k] <= tcull2)) t[k] = __int_as_float(0x7f800000);
            cswap(t[0], c[0], t[1], c[1]);
            cswap(t[2], c[2], t[3], c[3]);
            cswap(t[0], c[0], t[2], c[2]);
            cswap(t[1], c[1], t[3], c[3]);
            cswap(t[1], c[1], t[2], c[2]);
            const float inf = __int_as_float(0x7f800000);
            if (t[0] < inf) {
                const int pushes = (t[1] < inf) + (t[2] < inf) + (t[3] < inf);
                if (sp + pushes > kStack) {
                    err |= kErrWatchdogTraverse;
                    finished = true;
                    break;
                }
                if (t[3] < inf) push(sp++, c[3], t[3]);
                if (t[2] < inf) push(sp++, c[2], t[2]);
                if (t[1] < inf) push(sp++, c[1], t[1]);
                cur = c[0];
                continue;
            }
            bool found = false;
            while (sp > 0) {
                sp--;
                const float st_t = sp < kSmemStack ? s_t[sp][tid] : l_t[sp - kSmemStack];
                if (st_t <= ht * kCullMargin) {
                    cur = sp < kSmemStack ? s_node[sp][tid] : l_node[sp - kSmemStack];
                    found = true;
                    break;
                }
            }
            if (!found) finished = true;
        }
        if (finished) {
            q.hit[idx] = make_float4(__int_as_float(htri), hbu, hbv, hbw);
            if (q.perm) bin_cost_add(q, q.key[idx].x, visits);
            idx = kNeed;
        }
    }
    if (err) atomicOr(&ls.jobs[ls.job_ids[job_k]].state->err, err);
}

// each occupied slot's 32-byte record from its winner (after every photon of the pass is hashed,
// in all waves); one thread per hash slot of every job
__global__ void __launch_bounds__(256) k_slot_fill(LaunchSet ls) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ls.total) return;
    const int k = find_job(ls, g);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    const uint32_t slot = g - ls.prefix[k];
    uint32_t sidx = J.winner[slot];
    if (sidx == kEmptySlot) return;
    if (sidx == J.PW * J.PH) sidx = 0;  // every photon of the slot clipped: the cleared texel's photon 0
    const JobState* st = J.state;
    const float4 p = J.ph.pos[sidx], f = J.ph.flux[sidx], dd = J.ph.dir[sidx];
    const float G = st->grid_scale;
    const float fx = (p.x - st->bbmin[0]) * G, fy = (p.y - st->bbmin[1]) * G, fz = (p.z - st->bbmin[2]) * G;
    const float cx = floorf(fx), cy = floorf(fy), cz = floorf(fz);
    auto unorm16 = [](float x) { return (uint32_t)fminf(fmaxf(x * 65536.0f, 0.0f), 65535.0f); };
    auto snorm16 = [](float x) { return (uint32_t)(uint16_t)(int16_t)__float2int_rn(fminf(fmaxf(x, -1.0f), 1.0f) * 32767.0f); };
    const float fs = J.scene.flux_unscale_inv;
    const __half2 frg = __floats2half2_rn(f.x * fs, f.y * fs);
    const __half2 fb_ = __floats2half2_rn(f.z * fs, 0.0f);
    SlotRec r;
    r.w0 = make_uint4(((uint32_t)(uint16_t)(int16_t)cx) | ((uint32_t)(uint16_t)(int16_t)cy << 16),
                      ((uint32_t)(uint16_t)(int16_t)cz) | (min(J.count[slot], 65535u) << 16),
                      unorm16(fx - cx) | (unorm16(fy - cy) << 16), unorm16(fz - cz));
    r.w1 = make_uint4(*reinterpret_cast<const uint32_t*>(&frg), *reinterpret_cast<const uint32_t*>(&fb_),
                      snorm16(dd.x) | (snorm16(dd.y) << 16), snorm16(dd.z));
    J.slots[slot] = r;
}

// double-float arithmetic (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2): a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi) / 2, about 48 significant bits.  The operations are
// error-free transformations built from IEEE FP32 adds, multiplies and fmaf; the intrinsics keep
// the compiler from contracting or reassociating them.
__device__ __forceinline__ float2 df_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ float2 df_two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return make_float2(p, __fmaf_rn(a, b, -p));
}
// x * f
__device__ __forceinline__ float2 df_mul_f(float2 x, float f) {
    const float p = __fmul_rn(x.x, f);
    const float e = __fmaf_rn(x.y, f, __fmaf_rn(x.x, f, -p));
    return df_fast_two_sum(p, e);
}
// x + y
__device__ __forceinline__ float2 df_add(float2 x, float2 y) {
    const float2 s = df_two_sum(x.x, y.x);
    return df_fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(x.y, y.y)));
}

// AccumulatePhotons (progressive.fs:65-95) over EVERY photon within the radius, read from the
// counting-sort grid: the hit point visits the grid cells its sphere touches (with a margin of a
// fixed-point unit and 1e-4 of the radius beyond the rounding of the distance test), and counts
// the photons of each cell (the record's cell equals the visited one: a slot also holds the
// photons of other cells that hash to it) inside the radius and facing it.  Each counts once; the
// flux sums are exact (FP16 values as integers in units of 2^-24), so they depend neither on the
// order of the records within a slot nor on the cells' size.
__device__ __forceinline__ void grid_accumulate(const PhotonGrid& grid, uint32_t slot_base, uint32_t hash_num,
                                                const JobState* st, float gx, float gy, float gz, float R2f,
                                                float4 qn4, float& fx, float& fy, float& fz, float& M) {
    const int F = grid_frac_bits(st), Fc = grid_cell_bits(F, grid.shift);
    const float sF = grid_frac_scale(F);
    const float G = st->grid_scale;
    // the hit point in grid fixed point (exact products) and the radius in the same units; a
    // record's coordinate q stands for q + 0.5, and (q + 0.5) - u = q - (u - 0.5), both exact
    const float ux = __fmul_rn(gx, sF), uy = __fmul_rn(gy, sF), uz = __fmul_rn(gz, sF);
    const float vx = __fsub_rn(ux, 0.5f), vy = __fsub_rn(uy, 0.5f), vz = __fsub_rn(uz, 0.5f);
    const float rq2 = __fmul_rn(__fmul_rn(__fmul_rn(R2f, G), G), __fmul_rn(sF, sF));
    const float rq = sqrtf(rq2) * 1.0001f + 1.0f;
    auto lo = [&](float u) -> uint32_t {
        const float v = u - rq;
        return v > 0.0f ? (uint32_t)v >> Fc : 0u;
    };
    auto hi = [&](float u) -> uint32_t {
        const float v = u + rq;
        return (v < 2097150.0f ? (uint32_t)v : 2097150u) >> Fc;
    };
    const uint32_t x0 = lo(ux), y0 = lo(uy), z0 = lo(uz);
    const uint32_t nx = hi(ux) - x0 + 1u, ny = hi(uy) - y0 + 1u, nz = hi(uz) - z0 + 1u;
    // a radius up to the initial one spans at most 2 * 8 / 2 + 2 cells an axis; a hit point
    // outside the grid or a radius that is not finite gathers nothing
    const bool sane = ux >= 0.0f && uy >= 0.0f && uz >= 0.0f && rq < 4.0e6f && nx <= 64 && ny <= 64 && nz <= 64;
    const uint32_t ncell = sane ? nx * ny * nz : 0u;
    unsigned long long sr = 0, sg = 0, sb = 0;
    uint32_t m = 0;
    // the cells in x-fastest order; the next cell's record range is loaded while the current
    // cell's records are tested
    uint32_t cx = x0, cy = y0, cz = z0;
    uint32_t slot = grid_cell_slot(cx, cy, cz, hash_num);
    uint32_t beg = __ldg(&grid.ofs[slot_base + slot]), end = __ldg(&grid.ofs[slot_base + slot + 1]);
    for (uint32_t n = 0; n < ncell; n++) {
        uint32_t nxc = cx + 1u, nyc = cy, nzc = cz;
        if (nxc == x0 + nx) {
            nxc = x0;
            if (++nyc == y0 + ny) {
                nyc = y0;
                ++nzc;
            }
        }
        uint32_t nbeg = 0, nend = 0;
        if (n + 1 < ncell) {
            const uint32_t ns = grid_cell_slot(nxc, nyc, nzc, hash_num);
            nbeg = __ldg(&grid.ofs[slot_base + ns]);
            nend = __ldg(&grid.ofs[slot_base + ns + 1]);
        }
        for (uint32_t i = beg; i < end; i++) {
            const uint4 r = __ldg(&grid.rec[i]);
            const unsigned long long q = ((unsigned long long)r.y << 32) | r.x;
            const uint32_t qx = (uint32_t)q & kGridCoordNone, qy = (uint32_t)(q >> 21) & kGridCoordNone,
                           qz = (uint32_t)(q >> 42);
            if ((qx >> Fc) != cx || (qy >> Fc) != cy || (qz >> Fc) != cz) continue;
            const float dx = __fsub_rn((float)qx, vx), dy = __fsub_rn((float)qy, vy), dz = __fsub_rn((float)qz, vz);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            if (!(d2 < rq2)) continue;
            if (!(grid_oct8_dot(r.w >> 16, qn4.x, qn4.y, qn4.z) < 0.0f)) continue;
            sr += grid_half_fixed(r.z & 0xFFFFu);
            sg += grid_half_fixed(r.z >> 16);
            sb += grid_half_fixed(r.w & 0xFFFFu);
            m++;
        }
        cx = nxc, cy = nyc, cz = nzc;
        beg = nbeg, end = nend;
    }
    fx = __fmul_rn(__ull2float_rn(sr), 5.9604644775390625e-8f);  // * 2^-24 (exact)
    fy = __fmul_rn(__ull2float_rn(sg), 5.9604644775390625e-8f);
    fz = __fmul_rn(__ull2float_rn(sb), 5.9604644775390625e-8f);
    M = (float)m;
}

// The grid gather of a warp's 32 pixels (an 8x4 tile).  Neighbouring hit points visit mostly the
// same cells, so when every lane with a hit point belongs to the same job and the union of the
// lanes' cell boxes holds at most kCoopMaxCells cells (and at most four times the largest lane's
// box), the warp walks that union together: a lane per cell looks up the cells' record ranges in
// one round, a warp scan concatenates them, and the concatenated records are loaded and decoded in
// batches of 32 (a lane per record, the test that the record lies in its cell included) into
// shared memory, where every lane tests every record of the batch against its own hit point.  A
// lane accepts exactly the photons inside its radius (the union holds all of them, and each photon
// sits in one cell), so its sums equal its own walk's; otherwise every lane walks its own cells
// (grid_accumulate).  All 32 lanes call it.
constexpr uint32_t kCoopMaxCells = 128;

struct GridWarpSmem {
    // the union's cells that hold records, in walk order
    uint32_t cell_off[kCoopMaxCells + 1];  // first index in the concatenation of their records
    uint32_t cell_beg[kCoopMaxCells];      // first record
    uint32_t cell_x[kCoopMaxCells], cell_y[kCoopMaxCells], cell_z[kCoopMaxCells];  // coordinates
    float4 rec[32];                        // the batch: the position (cells' fixed point) + flux r|g
    uint32_t w[32];                        // flux b | direction
};

__device__ __forceinline__ void grid_gather_warp(const LaunchSet& ls, const uint32_t* slot_prefix,
                                                 const PhotonGrid& grid, bool live, uint32_t k_in, uint32_t p,
                                                 GridWarpSmem& sm, float& fx, float& fy, float& fz, float& M) {
    const unsigned full = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    bool has = false;
    uint32_t k = 0;
    float gx = 0.0f, gy = 0.0f, gz = 0.0f, R2f = 0.0f, vx = 0.0f, vy = 0.0f, vz = 0.0f, rq2 = 0.0f;
    float4 qn4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t x0 = 0xFFFFFFFFu, y0 = 0xFFFFFFFFu, z0 = 0xFFFFFFFFu, x1 = 0, y1 = 0, z1 = 0, own = 0;
    // the lane's sphere's box in fixed-point units (empty without a hit point)
    int bx0 = 0x7FFFFFFF, by0 = 0x7FFFFFFF, bz0 = 0x7FFFFFFF, bx1 = -1, by1 = -1, bz1 = -1;
    int Fc = 0;
    const JobState* st = nullptr;
    if (live) {
        k = k_in;
        const JobDesc& J = ls.jobs[ls.job_ids[k]];
        if ((J.flags & SPPM_FLAG_PHOTON_GRID) && J.px.tri[p] >= 0) {
            st = J.state;
            const bool f64 = (J.flags & SPPM_FLAG_FP64_STATISTICS) != 0;
            if (st->frame == 0) {
                R2f = f64 ? (float)((double)st->r0 * (double)st->r0) : __fmul_rn(st->r0, st->r0);
            } else if (f64) {
                R2f = (float)reinterpret_cast<const double*>(J.px.stat_r2)[p];
            } else {
                const float2 r2 = J.px.stat_r2[p];
                R2f = r2.x + r2.y;
            }
            const float G = st->grid_scale;
            const float4 qp4 = J.px.pos[p];
            qn4 = J.px.nrm[p];
            gx = __fmul_rn(fabsf(__fsub_rn(qp4.x, st->bbmin[0])), G);
            gy = __fmul_rn(fabsf(__fsub_rn(qp4.y, st->bbmin[1])), G);
            gz = __fmul_rn(fabsf(__fsub_rn(qp4.z, st->bbmin[2])), G);
            const int F = grid_frac_bits(st);
            Fc = grid_cell_bits(F, grid.shift);
            const float sF = grid_frac_scale(F);
            const float ux = __fmul_rn(gx, sF), uy = __fmul_rn(gy, sF), uz = __fmul_rn(gz, sF);
            vx = __fsub_rn(ux, 0.5f), vy = __fsub_rn(uy, 0.5f), vz = __fsub_rn(uz, 0.5f);
            rq2 = __fmul_rn(__fmul_rn(__fmul_rn(R2f, G), G), __fmul_rn(sF, sF));
            const float rq = sqrtf(rq2) * 1.0001f + 1.0f;
            if (ux >= 0.0f && uy >= 0.0f && uz >= 0.0f && rq < 4.0e6f) {
                has = true;
                bx0 = (int)floorf(vx - rq), by0 = (int)floorf(vy - rq), bz0 = (int)floorf(vz - rq);
                bx1 = (int)ceilf(vx + rq), by1 = (int)ceilf(vy + rq), bz1 = (int)ceilf(vz + rq);
                auto lo = [&](float u) -> uint32_t {
                    const float v = u - rq;
                    return v > 0.0f ? (uint32_t)v >> Fc : 0u;
                };
                auto hi = [&](float u) -> uint32_t {
                    const float v = u + rq;
                    return (v < 2097150.0f ? (uint32_t)v : 2097150u) >> Fc;
                };
                x0 = lo(ux), y0 = lo(uy), z0 = lo(uz), x1 = hi(ux), y1 = hi(uy), z1 = hi(uz);
                own = (x1 - x0 + 1u) * (y1 - y0 + 1u) * (z1 - z0 + 1u);
            }
        }
    }
    fx = fy = fz = M = 0.0f;
    const unsigned hasmask = __ballot_sync(full, has);
    if (!hasmask) return;
    const uint32_t kmin = __reduce_min_sync(full, has ? k : 0xFFFFFFFFu);
    const uint32_t kmax = __reduce_max_sync(full, has ? k : 0u);
    const uint32_t X0 = __reduce_min_sync(full, x0), Y0 = __reduce_min_sync(full, y0), Z0 = __reduce_min_sync(full, z0);
    const uint32_t X1 = __reduce_max_sync(full, x1), Y1 = __reduce_max_sync(full, y1), Z1 = __reduce_max_sync(full, z1);
    const uint32_t own_max = __reduce_max_sync(full, own);
    const uint32_t UX = X1 - X0 + 1u, UY = Y1 - Y0 + 1u, UZ = Z1 - Z0 + 1u;
    const unsigned long long ucells = (unsigned long long)UX * UY * UZ;
    if (kmin != kmax || ucells > 4ull * own_max || ucells > kCoopMaxCells) {
        if (has) {
            const JobDesc& J = ls.jobs[ls.job_ids[k]];
            grid_accumulate(grid, __ldg(&slot_prefix[k]), J.hash_num, st, gx, gy, gz, R2f, qn4, fx, fy, fz, M);
        }
        return;
    }
    // the warp's job (uniform)
    const JobDesc& J = ls.jobs[ls.job_ids[kmin]];
    const uint32_t slot_base = __ldg(&slot_prefix[kmin]), hash_num = J.hash_num, nc = (uint32_t)ucells;
    const int Fw = __shfl_sync(full, Fc, __ffs(hasmask) - 1);
    // a lane per cell (rounds of 32 cells): the record ranges, concatenated by a scan; the cells
    // without records are left out
    uint32_t run = 0, ne = 0;
    const unsigned below = (1u << lane) - 1u;
    for (uint32_t c0 = 0; c0 < nc; c0 += 32u) {
        const uint32_t c = c0 + lane;
        uint32_t b = 0, n = 0, cx = 0, cy = 0, cz = 0;
        if (c < nc) {
            const uint32_t t = c / UX;
            cx = X0 + (c - t * UX), cy = Y0 + t % UY, cz = Z0 + t / UY;
            const uint32_t slot = grid_cell_slot(cx, cy, cz, hash_num);
            b = __ldg(&grid.ofs[slot_base + slot]);
            n = __ldg(&grid.ofs[slot_base + slot + 1]) - b;
        }
        uint32_t incl = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(full, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        const unsigned held = __ballot_sync(full, n > 0);
        if (n > 0) {
            const uint32_t at = ne + __popc(held & below);
            sm.cell_off[at] = run + incl - n;
            sm.cell_beg[at] = b;
            sm.cell_x[at] = cx, sm.cell_y[at] = cy, sm.cell_z[at] = cz;
        }
        run += __shfl_sync(full, incl, 31);
        ne += __popc(held);
    }
    if (lane == 0) sm.cell_off[ne] = run;
    __syncwarp();
    // the box of the lanes' spheres: a record outside it is inside no lane's radius
    const int BX0 = __reduce_min_sync(full, bx0), BY0 = __reduce_min_sync(full, by0), BZ0 = __reduce_min_sync(full, bz0);
    const int BX1 = __reduce_max_sync(full, bx1), BY1 = __reduce_max_sync(full, by1), BZ1 = __reduce_max_sync(full, bz1);
    unsigned long long sr = 0, sg = 0, sb = 0;
    uint32_t m = 0;
    for (uint32_t base = 0; base < run; base += 32u) {
        const uint32_t g = base + lane;
        float4 ent = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        uint32_t w = 0;
        bool keep = false;
        if (g < run) {
            // the cell of concatenation index g: the last cell starting at or before g
            uint32_t lo = 0, hi = ne - 1u;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1u) >> 1;
                if (sm.cell_off[mid] <= g) lo = mid;
                else hi = mid - 1u;
            }
            const uint32_t cx = sm.cell_x[lo], cy = sm.cell_y[lo], cz = sm.cell_z[lo];
            const uint4 r = __ldg(&grid.rec[sm.cell_beg[lo] + (g - sm.cell_off[lo])]);
            const unsigned long long q = ((unsigned long long)r.y << 32) | r.x;
            const uint32_t qx = (uint32_t)q & kGridCoordNone, qy = (uint32_t)(q >> 21) & kGridCoordNone,
                           qz = (uint32_t)(q >> 42);
            keep = (qx >> Fw) == cx && (qy >> Fw) == cy && (qz >> Fw) == cz && (int)qx >= BX0 && (int)qx <= BX1 &&
                   (int)qy >= BY0 && (int)qy <= BY1 && (int)qz >= BZ0 && (int)qz <= BZ1;
            ent = make_float4((float)qx, (float)qy, (float)qz, __uint_as_float(r.z));
            w = r.w;
        }
        // the batch's records that may lie inside some lane's radius, packed to the front
        const unsigned kept = __ballot_sync(full, keep);
        if (keep) {
            const uint32_t at = __popc(kept & ((1u << lane) - 1u));
            sm.rec[at] = ent;
            sm.w[at] = w;
        }
        __syncwarp();
        const uint32_t n = __popc(kept);
        if (has) {
#pragma unroll 2
            for (uint32_t j = 0; j < n; j++) {
                const float4 c = sm.rec[j];
                const float dx = __fsub_rn(c.x, vx), dy = __fsub_rn(c.y, vy), dz = __fsub_rn(c.z, vz);
                const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                if (!(d2 < rq2)) continue;
                const uint32_t ww = sm.w[j];
                if (!(grid_oct8_dot(ww >> 16, qn4.x, qn4.y, qn4.z) < 0.0f)) continue;
                const uint32_t rz = __float_as_uint(c.w);
                sr += grid_half_fixed(rz & 0xFFFFu);
                sg += grid_half_fixed(rz >> 16);
                sb += grid_half_fixed(ww & 0xFFFFu);
                m++;
            }
        }
        __syncwarp();
    }
    fx = __fmul_rn(__ull2float_rn(sr), 5.9604644775390625e-8f);  // * 2^-24 (exact)
    fy = __fmul_rn(__ull2float_rn(sg), 5.9604644775390625e-8f);
    fz = __fmul_rn(__ull2float_rn(sb), 5.9604644775390625e-8f);
    M = (float)m;
}

// progressive.fs with the slot records (or, for jobs with SPPM_FLAG_PHOTON_GRID, every photon of
// the counting-sort grid), FP32 flux gathering and double-float statistics (ANY_F64: the variant
// launched when some job of the launch keeps IEEE double statistics; ANY_GRID: when some job uses
// the grid; slot_prefix: the hash-slot launch set's prefix sums)
template <bool ANY_F64, bool ANY_GRID>
__global__ void __launch_bounds__(256) k_gather_mixed(LaunchSet ls, const uint32_t* slot_prefix, PhotonGrid grid) {
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = gi < ls.total;
    int k = 0;
    uint32_t p = 0;
    if (live) {
        k = find_job(ls, gi);
        p = gi - ls.prefix[k];
        if (ANY_GRID) {
            // the launch covers each job in 8x4-pixel tiles, a warp per tile (neighbouring hit points)
            const JobDesc& Jt = ls.jobs[ls.job_ids[k]];
            const uint32_t tw = (Jt.W + 7u) >> 3, tile = p >> 5, lane = p & 31u;
            const uint32_t px = (tile % tw) * 8u + (lane & 7u), py = (tile / tw) * 4u + (lane >> 3);
            live = px < Jt.W && py < Jt.H;
            p = py * Jt.W + px;
        }
    }
    float gfx = 0.0f, gfy = 0.0f, gfz = 0.0f, gM = 0.0f;
    if (ANY_GRID) {
        __shared__ GridWarpSmem s_grid[256 / 32];
        grid_gather_warp(ls, slot_prefix, grid, live, (uint32_t)k, p, s_grid[threadIdx.x >> 5], gfx, gfy, gfz, gM);
    }
    if (!live) return;
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    JobState* st = J.state;
    const uint32_t frame = st->frame;
    if (p == 0) {
        const uint32_t e = st->emitted_frame;
        st->num_photons_f32 = __fadd_rn(st->num_photons_f32, (float)(int)e);
        st->num_photons += e;
        st->photon_segments += st->segments_frame;
    }
    const float2 zero = make_float2(0.0f, 0.0f);
    // the statistics' 8-byte words hold double-float pairs, or IEEE doubles for jobs with
    // SPPM_FLAG_FP64_STATISTICS
    const bool f64 = ANY_F64 && (J.flags & SPPM_FLAG_FP64_STATISTICS) != 0;
    float2 N = zero, R2 = zero, tx = zero, ty = zero, tz = zero;
    double R2d64 = 0.0, T64[3] = {0.0, 0.0, 0.0};
    if (f64) {
        R2d64 = frame == 0 ? (double)st->r0 * (double)st->r0 : reinterpret_cast<const double*>(J.px.stat_r2)[p];
        if (frame != 0) {
            const double* Td = reinterpret_cast<const double*>(J.px.stat_tau) + 3 * (size_t)p;
            T64[0] = Td[0], T64[1] = Td[1], T64[2] = Td[2];
        }
        R2 = make_float2((float)R2d64, 0.0f);
        N = make_float2((float)reinterpret_cast<const double*>(J.px.stat_n)[p], 0.0f);
    } else {
        N = J.px.stat_n[p];
        R2 = frame == 0 ? df_two_prod(st->r0, st->r0) : J.px.stat_r2[p];
        tx = frame == 0 ? zero : J.px.stat_tau[3 * (size_t)p + 0];
        ty = frame == 0 ? zero : J.px.stat_tau[3 * (size_t)p + 1];
        tz = frame == 0 ? zero : J.px.stat_tau[3 * (size_t)p + 2];
    }
    if (J.px.tri[p] >= 0) {
        const float G = st->grid_scale;
        const float hs1 = st->hash_scale1;
        const float hn = (float)J.hash_num;
        const float4 qp4 = J.px.pos[p], qn4 = J.px.nrm[p], qr4 = J.px.refl[p];
        const float gx = __fmul_rn(fabsf(__fsub_rn(qp4.x, st->bbmin[0])), G),
                    gy = __fmul_rn(fabsf(__fsub_rn(qp4.y, st->bbmin[1])), G),
                    gz = __fmul_rn(fabsf(__fsub_rn(qp4.z, st->bbmin[2])), G);
        const float ix = floorf(gx - 0.5f), iy = floorf(gy - 0.5f), iz = floorf(gz - 0.5f);
        const float R2f = R2.x + R2.y;  // the in-radius test in FP32
        const float invG = 1.0f / G;
        float fx = 0.0f, fy = 0.0f, fz = 0.0f, M = 0.0f;
        if (ANY_GRID && (J.flags & SPPM_FLAG_PHOTON_GRID)) {
            fx = gfx, fy = gfy, fz = gfz, M = gM;
        } else {
        uint32_t slots[8];
        hash_cells8(mk(ix, iy, iz), G, hs1, hn, slots);
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const float cx = ix + (float)(c & 1), cy = iy + (float)((c >> 1) & 1), cz = iz + (float)(c >> 2);
            const uint32_t slot = slots[c];
            const SlotRec r = J.slots[slot];
            const uint32_t cnt = r.w0.y >> 16;
            if (cnt == 0 || J.winner[slot] == kEmptySlot) continue;
            if ((int)(int16_t)(r.w0.x & 0xFFFF) != (int)cx || (int)(int16_t)(r.w0.x >> 16) != (int)cy ||
                (int)(int16_t)(r.w0.y & 0xFFFF) != (int)cz)
                continue;  // the slot holds a photon of another cell (hash collision)
            const float px = (cx + (float)(r.w0.z & 0xFFFF) * (1.0f / 65536.0f)) * invG + st->bbmin[0];
            const float py = (cy + (float)(r.w0.z >> 16) * (1.0f / 65536.0f)) * invG + st->bbmin[1];
            const float pz = (cz + (float)(r.w0.w & 0xFFFF) * (1.0f / 65536.0f)) * invG + st->bbmin[2];
            const float dx = px - qp4.x, dy = py - qp4.y, dz = pz - qp4.z;
            if (dx * dx + dy * dy + dz * dz >= R2f) continue;
            const float ddx = (float)(int16_t)(r.w1.z & 0xFFFF), ddy = (float)(int16_t)(r.w1.z >> 16),
                        ddz = (float)(int16_t)(r.w1.w & 0xFFFF);
            if (!(qn4.x * ddx + qn4.y * ddy + qn4.z * ddz < 0.0f)) continue;
            const float2 frg = __half22float2(*reinterpret_cast<const __half2*>(&r.w1.x));
            const float2 fb_ = __half22float2(*reinterpret_cast<const __half2*>(&r.w1.y));
            const float cf = (float)cnt;
            fx += frg.x * cf;
            fy += frg.y * cf;
            fz += fb_.x * cf;
            M += cf;
        }
        }
        const float s = J.scene.flux_unscale * 0.318309886f;
        if (f64) {
            // IEEE double statistics: the shrink ratio (N + alpha M) / (N + M), N, R^2 and tau in
            // FP64 arithmetic (the FP32 flux sums enter once, rounded to double exactly)
            double* Nd = reinterpret_cast<double*>(J.px.stat_n) + p;
            double* R2d = reinterpret_cast<double*>(J.px.stat_r2) + p;
            double* Td = reinterpret_cast<double*>(J.px.stat_tau) + 3 * (size_t)p;
            const double n0 = *Nd, m = (double)M, a = (double)J.alpha;
            const double ratio = M > 0.0f ? fmin((n0 + a * m) / (n0 + m), 1.0) : 1.0;
            *R2d = R2d64 * ratio;
            *Nd = fma(a, m, n0);
            const double fs = (double)s;
            Td[0] = (T64[0] + (double)fx * fs * (double)qr4.x) * ratio;
            Td[1] = (T64[1] + (double)fy * fs * (double)qr4.y) * ratio;
            Td[2] = (T64[2] + (double)fz * fs * (double)qr4.z) * ratio;
            return;
        }
        // shrink ratio (N + alpha M) / (N + M) = 1 - (1 - alpha) M / (N + M), computed in FP32 (its
        // relative error ~1e-7 per pass); the statistics accumulate in double-float
        const float denom = (N.x + N.y) + M;
        const float ggf = M > 0.0f ? fminf(1.0f - (1.0f - J.alpha) * (M / denom), 1.0f) : 1.0f;
        R2 = df_mul_f(R2, ggf);
        N = df_add(N, df_two_prod(J.alpha, M));
        tx = df_add(df_mul_f(tx, ggf), make_float2(fx * s * qr4.x * ggf, 0.0f));
        ty = df_add(df_mul_f(ty, ggf), make_float2(fy * s * qr4.y * ggf, 0.0f));
        tz = df_add(df_mul_f(tz, ggf), make_float2(fz * s * qr4.z * ggf, 0.0f));
        J.px.stat_n[p] = N;
    }
    if (f64) {
        reinterpret_cast<double*>(J.px.stat_r2)[p] = R2d64;
        double* Td = reinterpret_cast<double*>(J.px.stat_tau) + 3 * (size_t)p;
        Td[0] = T64[0], Td[1] = T64[1], Td[2] = T64[2];
        return;
    }
    J.px.stat_r2[p] = R2;
    J.px.stat_tau[3 * (size_t)p + 0] = tx;
    J.px.stat_tau[3 * (size_t)p + 1] = ty;
    J.px.stat_tau[3 * (size_t)p + 2] = tz;
}

// re.fs from the statistics (the image is FP32: the pairs' high parts, or the doubles, carry it)
__global__ void k_resolve_mixed(LaunchSet ls, uint32_t display) {
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= ls.total) return;
    const int k = find_job(ls, gi);
    const JobDesc& J = ls.jobs[ls.job_ids[k]];
    const uint32_t p = gi - ls.prefix[k];
    const bool f64 = (J.flags & SPPM_FLAG_FP64_STATISTICS) != 0;
    const float2 r2 = J.px.stat_r2[p];
    const float r2f = f64 ? (float)reinterpret_cast<const double*>(J.px.stat_r2)[p] : r2.x + r2.y;
    const float den = r2f * 3.14159265f * (float)J.state->num_photons;
    const float4 qe = J.px.emi_n[p];
    const float e[3] = {qe.x, qe.y, qe.z};
    for (int c = 0; c < 3; c++) {
        const float2 t = J.px.stat_tau[3 * (size_t)p + c];
        const float tf = f64 ? (float)reinterpret_cast<const double*>(J.px.stat_tau)[3 * (size_t)p + c] : t.x + t.y;
        float v = tf / den + e[c];
        if (display) {
            v = 1.0f - sppm_fexp(-v * 60000.0f);
            v = v < 0.0031308f ? 12.92f * v : 1.055f * sppm_fpow(v, 0.416666666667f) - 0.055f;
        }
        J.image[(size_t)p * 3 + c] = v;
    }
}

static inline uint32_t blocks_for(uint32_t n, uint32_t b) { return (n + b - 1) / b; }

void launch_trace_photons4(const LaunchSet& ls, const RayQueue& q, uint32_t persistent_blocks, cudaStream_t s) {
    if (ls.total) k_trace_photons4<<<persistent_blocks, kTraceBlock, 0, s>>>(ls, q);
}
uint32_t trace_photons4_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace_photons4, kTraceBlock, 0) != cudaSuccess) n = 4;
    return n > 0 ? (uint32_t)n : 1u;
}
void launch_slot_fill(const LaunchSet& hash_slots, cudaStream_t s) {
    if (hash_slots.total) k_slot_fill<<<blocks_for(hash_slots.total, 256), 256, 0, s>>>(hash_slots);
}
void launch_gather_mixed(const LaunchSet& ls, uint32_t block, bool any_fp64, const uint32_t* slot_prefix,
                         const PhotonGrid* grid, cudaStream_t s) {
    const uint32_t b = block >= 32 && block <= 256 && block % 32 == 0 ? block : 256;
    if (!ls.total) return;
    const PhotonGrid g = grid ? *grid : PhotonGrid{};
    const uint32_t n = blocks_for(ls.total, b);
    if (grid) {
        if (any_fp64) k_gather_mixed<true, true><<<n, b, 0, s>>>(ls, slot_prefix, g);
        else k_gather_mixed<false, true><<<n, b, 0, s>>>(ls, slot_prefix, g);
    } else {
        if (any_fp64) k_gather_mixed<true, false><<<n, b, 0, s>>>(ls, slot_prefix, g);
        else k_gather_mixed<false, false><<<n, b, 0, s>>>(ls, slot_prefix, g);
    }
}
void launch_resolve_mixed(const LaunchSet& ls, uint32_t display, cudaStream_t s) {
    if (ls.total) k_resolve_mixed<<<blocks_for(ls.total, 256), 256, 0, s>>>(ls, display);
}

}  // namespace sppm_dev

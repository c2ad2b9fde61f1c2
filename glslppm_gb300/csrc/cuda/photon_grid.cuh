// Counting-sort photon grid of the mixed path (SPPM_FLAG_PHOTON_GRID): record format and the
// arithmetic the scatter and the gather share.
//
// Instead of one winning photon per hash slot and the slot's count (scatter.vs:15-23,
// correction.vs) the grid keeps every stored photon, sorted by slot: the store's insertion counts
// the slot's photons and hands each photon its rank among them, an exclusive scan turns the
// counts into offsets, and a scatter writes one 16-byte record per photon at offset(slot) + rank.
// The gather (progressive.fs:98-142 with AccumulatePhotons :65-95 summed over every photon) visits
// the cells that the sphere of the hit point's radius touches and reads their slots' contiguous
// records.  The grid's cells are the reference's (hash.fs:51-68: 1 / GridScale = twice the
// initial radius) split 2^shift times along each axis (sppm_tuning.grid_cell_shift), hashed by an
// integer hash; the photons a hit point gathers -- every photon inside its radius -- and so every
// result are the same for any shift.
//
// Record (uint4):
//   x, y  the position as three 21-bit grid fixed-point coordinates q = floor(u * 2^F), u = (p -
//         BBoxMin) * GridScale (hash.fs's cell coordinate before its floor, so q >> F is the cell),
//         packed x | y << 21 | z << 42 into a 64-bit word, low word first (a photon with a
//         coordinate outside [0, 2^21 - 1) is outside the grid: no hit point's radius reaches it,
//         and it gets no record)
//   z     flux r | g << 16 (FP16 of flux / (light area * pi), at most 65504)
//   w     flux b | octahedral direction x << 16 | y << 24 (signed 8-bit, scale 127)
// F = 21 - bits(cells + 1), cells = the reference grid's largest cell count along an axis, so that
// every cell index inside the grid is below the all-ones value; a grid cell is q >> (F - shift).
//
// The arithmetic is written with round-to-nearest intrinsics and no contraction: the CPU
// restatement (oracle/sppm_oracle.c, single-precision build) computes the same records and the
// same gathered counts and flux sums.
#pragma once

#include <cuda_fp16.h>

#include "device_common.cuh"

namespace sppm_dev {

constexpr uint32_t kGridCoordBits = 21;
constexpr uint32_t kGridCoordNone = (1u << kGridCoordBits) - 1;  // all ones: outside the grid
constexpr uint32_t kGridScanBlock = 256;
constexpr uint32_t kGridScanItems = 8;
constexpr uint32_t kGridTile = kGridScanBlock * kGridScanItems;  // hash slots per scan tile

// fraction bits F of a job's grid fixed point, from the frame state the store used
__device__ __forceinline__ int grid_frac_bits(const JobState* st) {
    uint32_t cells = 0;
    for (int c = 0; c < 3; c++) {
        const float e = __fmul_rn(__fsub_rn(st->bbmax[c], st->bbmin[c]), st->grid_scale);
        const uint32_t n = e > 0.0f ? (e < 2097152.0f ? (uint32_t)ceilf(e) : 2097152u) : 0u;
        cells = n > cells ? n : cells;
    }
    const int b = 32 - __clz((int)(cells + 1u));
    return b < (int)kGridCoordBits ? (int)kGridCoordBits - b : 0;
}

// 2^F as a float (exact)
__device__ __forceinline__ float grid_frac_scale(int F) { return __int_as_float((127 + F) << 23); }

// grid fixed-point coordinate of one position component
__device__ __forceinline__ uint32_t grid_coord(float p, float bbmin, float G, float sF) {
    const float v = __fmul_rn(__fmul_rn(__fsub_rn(p, bbmin), G), sF);  // the second product is exact
    return v >= 0.0f && v < 2097151.0f ? (uint32_t)v : kGridCoordNone;  // truncation = floor here
}

// two signed 8-bit octahedral components of a direction (Meyer et al., "On floating-point
// normal vectors", EGSR 2010: project onto |x|+|y|+|z| = 1, fold the lower hemisphere)
__device__ __forceinline__ uint32_t grid_oct8(float x, float y, float z) {
    const float s = __fadd_rn(__fadd_rn(fabsf(x), fabsf(y)), fabsf(z));
    if (!(s > 0.0f)) return 0u;
    float ox = __fdiv_rn(x, s), oy = __fdiv_rn(y, s);
    if (z < 0.0f) {
        const float tx = __fmul_rn(__fsub_rn(1.0f, fabsf(oy)), copysignf(1.0f, ox));
        const float ty = __fmul_rn(__fsub_rn(1.0f, fabsf(ox)), copysignf(1.0f, oy));
        ox = tx;
        oy = ty;
    }
    const int a = __float2int_rn(__fmul_rn(ox, 127.0f)), b = __float2int_rn(__fmul_rn(oy, 127.0f));
    return ((uint32_t)a & 0xFFu) | (((uint32_t)b & 0xFFu) << 8);
}

// dot(n, d) for the (unnormalised) direction d an octahedral code stands for: its sign is what
// the gather's facing test reads; the decoded components are small integers (exact)
__device__ __forceinline__ float grid_oct8_dot(uint32_t code, float nx, float ny, float nz) {
    float x = (float)(int)(int8_t)(code & 0xFFu), y = (float)(int)(int8_t)((code >> 8) & 0xFFu);
    const float ax = fabsf(x), ay = fabsf(y);
    const float z = 127.0f - ax - ay;
    if (z < 0.0f) {
        const float tx = (127.0f - ay) * copysignf(1.0f, x);
        y = (127.0f - ax) * copysignf(1.0f, y);
        x = tx;
    }
    return __fadd_rn(__fadd_rn(__fmul_rn(nx, x), __fmul_rn(ny, y)), __fmul_rn(nz, z));
}

__device__ __forceinline__ uint32_t grid_half(float v) {
    return (uint32_t)__half_as_ushort(__float2half_rn(fminf(v, 65504.0f)));
}

// a photon's record (pos, flux and dir as the store left them)
__device__ __forceinline__ uint4 grid_record(const JobDesc& J, const JobState* st, int F, float4 p, float4 f,
                                             float4 d) {
    const float G = st->grid_scale, sF = grid_frac_scale(F);
    const uint64_t qx = grid_coord(p.x, st->bbmin[0], G, sF), qy = grid_coord(p.y, st->bbmin[1], G, sF),
                   qz = grid_coord(p.z, st->bbmin[2], G, sF);
    const uint64_t q = qx | (qy << 21) | (qz << 42);
    const float fs = J.scene.flux_unscale_inv;
    const uint32_t hr = grid_half(__fmul_rn(f.x, fs)), hg = grid_half(__fmul_rn(f.y, fs)),
                   hb = grid_half(__fmul_rn(f.z, fs));
    return make_uint4((uint32_t)q, (uint32_t)(q >> 32), hr | (hg << 16), hb | (grid_oct8(d.x, d.y, d.z) << 16));
}

// fraction bits of a grid cell: F less the cell split (at most F)
__device__ __forceinline__ int grid_cell_bits(int F, uint32_t shift) { return F - min((int)shift, F); }

// the hash slot of a grid cell (Teschner et al., "Optimized Spatial Hashing for Collision
// Detection of Deformable Objects", VMV 2003, reduced to [0, n) by a multiply-high)
__device__ __forceinline__ uint32_t grid_cell_slot(uint32_t cx, uint32_t cy, uint32_t cz, uint32_t n) {
    return __umulhi((cx * 73856093u) ^ (cy * 19349663u) ^ (cz * 83492791u), n);
}

// the hash slot of a stored photon at p, or 0xFFFFFFFF when p is outside the grid (no record)
__device__ __forceinline__ uint32_t grid_photon_slot(const JobDesc& J, const JobState* st, uint32_t shift, float px,
                                                     float py, float pz) {
    const int F = grid_frac_bits(st), Fc = grid_cell_bits(F, shift);
    const float G = st->grid_scale, sF = grid_frac_scale(F);
    const uint32_t qx = grid_coord(px, st->bbmin[0], G, sF), qy = grid_coord(py, st->bbmin[1], G, sF),
                   qz = grid_coord(pz, st->bbmin[2], G, sF);
    if (qx == kGridCoordNone || qy == kGridCoordNone || qz == kGridCoordNone) return 0xFFFFFFFFu;
    return grid_cell_slot(qx >> Fc, qy >> Fc, qz >> Fc, J.hash_num);
}

// value * 2^24 of a finite, non-negative FP16 (exact; at most 65504 * 2^24 < 2^40)
__device__ __forceinline__ uint64_t grid_half_fixed(uint32_t h) {
    const uint32_t e = (h >> 10) & 31u, m = h & 1023u;
    return e ? (uint64_t)(m | 1024u) << (e - 1u) : (uint64_t)m;
}

}  // namespace sppm_dev

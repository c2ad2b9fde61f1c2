// Counting-sort photon grid (SPPM_FLAG_PHOTON_GRID): the exclusive scan of the hash slots' photon
// counts over every job of a launch and the scatter of the photon records (photon_grid.cuh).
//
// The counts and each photon's rank within its slot come from the photon store's hash insertion
// (warp-aggregated: one atomic per warp and slot).  The scan is the three-phase tiled form --
// tile sums, one block scanning them, then each tile scanned with its offset -- in 2048-slot
// tiles: no block waits on another.  The scatter writes each stored photon's record at
// offset(slot) + rank, so the records of a slot are contiguous and the records of a job follow
// the previous job's.
#include <cstdint>

#include "device_common.cuh"
#include "kernels.h"
#include "photon_grid.cuh"

namespace sppm_dev {

namespace {

// count of the launch's global hash slot g (0 beyond the end)
__device__ __forceinline__ uint32_t grid_slot_count(const LaunchSet& hs, uint32_t g) {
    if (g >= hs.total) return 0u;
    const int k = find_job(hs, g);
    const JobDesc& J = hs.jobs[hs.job_ids[k]];
    return J.count[g - hs.prefix[k]];
}

// exclusive scan of one value per thread of a kGridScanBlock-thread block; *total = the block's sum
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= (uint32_t)d) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    constexpr uint32_t kWarps = kGridScanBlock / 32;
    if (warp == 0) {
        uint32_t w = lane < kWarps ? warp_sums[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, d);
            if (lane >= (uint32_t)d) w += y;
        }
        if (lane < kWarps) warp_sums[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[kWarps - 1];
    return before + x - v;
}

// the tile's counts into shared memory, read in coalesced stripes; returns the thread's
// kGridScanItems consecutive counts' sum (items t * kGridScanItems ..)
__device__ __forceinline__ uint32_t load_tile(const LaunchSet& hs, uint32_t* s_cnt) {
    const uint32_t base = blockIdx.x * kGridTile;
#pragma unroll
    for (uint32_t j = 0; j < kGridScanItems; j++) {
        const uint32_t i = j * kGridScanBlock + threadIdx.x;
        s_cnt[i + (i >> 5)] = grid_slot_count(hs, base + i);  // one pad word per 32: no bank conflicts
    }
    __syncthreads();
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t j = 0; j < kGridScanItems; j++) {
        const uint32_t i = threadIdx.x * kGridScanItems + j;
        sum += s_cnt[i + (i >> 5)];
    }
    return sum;
}

constexpr uint32_t kPaddedTile = kGridTile + kGridTile / 32;

__global__ void __launch_bounds__(kGridScanBlock) k_grid_tile_sums(LaunchSet hs, PhotonGrid grid) {
    __shared__ uint32_t s_cnt[kPaddedTile];
    __shared__ uint32_t s_warp[kGridScanBlock / 32];
    const uint32_t sum = load_tile(hs, s_cnt);
    uint32_t total;
    block_exclusive_scan(sum, s_warp, &total);
    if (threadIdx.x == 0) grid.tile_sums[blockIdx.x] = total;
}

// one block: the tile sums -> their exclusive prefix sums, in chunks; ofs[total] = the sum of all
__global__ void __launch_bounds__(kGridScanBlock) k_grid_tile_scan(LaunchSet hs, PhotonGrid grid) {
    __shared__ uint32_t s_warp[kGridScanBlock / 32];
    uint32_t carry = 0;
    for (uint32_t c = 0; c < grid.tiles; c += kGridScanBlock) {
        const uint32_t i = c + threadIdx.x;
        const uint32_t v = i < grid.tiles ? grid.tile_sums[i] : 0u;
        uint32_t total;
        const uint32_t ex = block_exclusive_scan(v, s_warp, &total);
        if (i < grid.tiles) grid.tile_sums[i] = carry + ex;
        carry += total;
        __syncthreads();  // s_warp is reused by the next chunk
    }
    if (threadIdx.x == 0) grid.ofs[hs.total] = carry;
}

__global__ void __launch_bounds__(kGridScanBlock) k_grid_offsets(LaunchSet hs, PhotonGrid grid) {
    __shared__ uint32_t s_cnt[kPaddedTile];
    __shared__ uint32_t s_warp[kGridScanBlock / 32];
    const uint32_t sum = load_tile(hs, s_cnt);
    uint32_t total;
    uint32_t run = grid.tile_sums[blockIdx.x] + block_exclusive_scan(sum, s_warp, &total);
#pragma unroll
    for (uint32_t j = 0; j < kGridScanItems; j++) {
        const uint32_t i = threadIdx.x * kGridScanItems + j;
        const uint32_t c = s_cnt[i + (i >> 5)];
        s_cnt[i + (i >> 5)] = run;
        run += c;
    }
    __syncthreads();
    const uint32_t base = blockIdx.x * kGridTile;
#pragma unroll
    for (uint32_t j = 0; j < kGridScanItems; j++) {
        const uint32_t i = j * kGridScanBlock + threadIdx.x;
        if (base + i < hs.total) grid.ofs[base + i] = s_cnt[i + (i >> 5)];
    }
}

// one thread per photon slot of the launch: the record of each photon stored this pass (flux
// >= 0; terminated and unstored photons carry a negative flux) at offset(slot) + rank (below the
// record capacity by construction: the check keeps a write in bounds whatever the keys hold)
__global__ void __launch_bounds__(256) k_grid_scatter(LaunchSet ph, const uint32_t* slot_prefix, PhotonGrid grid) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ph.total) return;
    const int k = find_job(ph, g);
    const JobDesc& J = ph.jobs[ph.job_ids[k]];
    if (!(J.flags & SPPM_FLAG_PHOTON_GRID)) return;
    const uint32_t sidx = g - ph.prefix[k];
    const float4 f = J.ph.flux[sidx];
    if (f.x < 0.0f) return;  // the store's test (photon_store)
    const JobState* st = J.state;
    const uint4 r = grid_record(J, st, grid_frac_bits(st), J.ph.pos[sidx], f, J.ph.dir[sidx]);
    // a photon outside the grid was not inserted (its key is not of this pass)
    const unsigned long long q = ((unsigned long long)r.y << 32) | r.x;
    if ((q & kGridCoordNone) == kGridCoordNone || ((q >> 21) & kGridCoordNone) == kGridCoordNone ||
        (q >> 42) == kGridCoordNone)
        return;
    const uint2 key = J.grid_key[sidx];
    const uint32_t at = grid.ofs[__ldg(&slot_prefix[k]) + key.x] + key.y;
    if (at < grid.rec_capacity) grid.rec[at] = r;
}

inline uint32_t blocks_for(uint32_t n, uint32_t b) { return (n + b - 1) / b; }

}  // namespace

uint32_t grid_tiles(uint32_t hash_slots) { return blocks_for(hash_slots, kGridTile); }

void launch_grid_sort(const LaunchSet& hash_slots, const LaunchSet& photons, const PhotonGrid& grid, cudaStream_t s) {
    if (!hash_slots.total || !grid.tiles) return;
    k_grid_tile_sums<<<grid.tiles, kGridScanBlock, 0, s>>>(hash_slots, grid);
    k_grid_tile_scan<<<1, kGridScanBlock, 0, s>>>(hash_slots, grid);
    k_grid_offsets<<<grid.tiles, kGridScanBlock, 0, s>>>(hash_slots, grid);
    if (photons.total) k_grid_scatter<<<blocks_for(photons.total, 256), 256, 0, s>>>(photons, hash_slots.prefix, grid);
}

}  // namespace sppm_dev

// Launchers of the SPPM kernels (host side).
#pragma once

#include <cuda_runtime.h>

#include "device_common.cuh"

namespace sppm_dev {

// the JobStates of up to kStateGatherMax job slots copied into out[0..n) (kernel parameter)
constexpr uint32_t kStateGatherMax = 256;
struct StateGather {
    uint32_t n;
    uint32_t slot[kStateGatherMax];
};
void launch_gather_states(const JobDesc* jobs, const StateGather& list, JobState* out, cudaStream_t s);

// bytes (a multiple of 8) from page-locked host memory mapped into the device's address space to
// device memory, by one block (a small upload without a copy-engine transfer)
void launch_copy_from_host(void* dst, const void* src_mapped, size_t bytes, cudaStream_t s);

// up to kDescCopyMax job descriptors from mapped staging slots to the runner's table, one block
// per descriptor, in one launch (kernel parameter)
constexpr uint32_t kDescCopyMax = 128;
struct DescCopy {
    uint32_t n;
    JobDesc* dst[kDescCopyMax];
    const JobDesc* src[kDescCopyMax];
};
void launch_copy_descs(const DescCopy& list, cudaStream_t s);

// plain FP32 path (kernels_fp32.cu)
void launch_frame_begin(const LaunchSet& ls, const RayQueue& q, cudaStream_t s);
// mixed: 4-wide BVH traversal; textured: some job of the launch has texture coordinates (the
// kernel variants with texture lookups)
// block: threads per block (a multiple of 32 up to the kernel's launch bound; 0 = the bound)
void launch_eye(const LaunchSet& ls, const RayQueue& q, bool mixed, bool textured, uint32_t block, cudaStream_t s);
void launch_grid(const JobDesc* jobs, const uint32_t* job_ids, uint32_t njobs, cudaStream_t s);
// the plain path's table of in-cell bounds for the grid launch_grid has just set
void launch_cell_bounds(const JobDesc* jobs, const uint32_t* job_ids, uint32_t njobs, cudaStream_t s);
void launch_photon_fp32(const LaunchSet& ls, bool count_traversal, bool textured, cudaStream_t s);
void launch_photon_gen_fp32(const LaunchSet& ls, const RayQueue& q, bool textured, cudaStream_t s);
void launch_queue_reset(const RayQueue& q, cudaStream_t s);
void launch_trace_photons_fp32(const LaunchSet& ls, const RayQueue& q, bool count_traversal,
                               uint32_t persistent_blocks, cudaStream_t s);
void launch_ray_bins(const RayQueue& q, cudaStream_t s);
// the bins' traversal order from the walks traced since the last call (longest mean first)
void launch_ray_bins_order(const RayQueue& q, cudaStream_t s);
void launch_trace_photons_coop(const LaunchSet& ls, const RayQueue& q, bool count_traversal, cudaStream_t s);
// grid_shift: the counting-sort grid's cell split (log2) for jobs with SPPM_FLAG_PHOTON_GRID
void launch_photon_store_fp32(const LaunchSet& ls, const RayQueue& q, uint32_t block, uint32_t grid_shift,
                              cudaStream_t s);
uint32_t trace_photons_blocks_per_sm();

// mixed-precision path (kernels_mixed.cu)
void launch_trace_photons4(const LaunchSet& ls, const RayQueue& q, uint32_t persistent_blocks, cudaStream_t s);
uint32_t trace_photons4_blocks_per_sm();
void launch_slot_fill(const LaunchSet& hash_slots, cudaStream_t s);
// grid: the launch's counting-sort photon grid when some job has SPPM_FLAG_PHOTON_GRID (else null),
// and then ls covers the pixels in 8x4 tiles (a warp per tile); slot_prefix: the hash-slot launch
// set's prefix sums
void launch_gather_mixed(const LaunchSet& ls, uint32_t block, bool any_fp64, const uint32_t* slot_prefix,
                         const PhotonGrid* grid, cudaStream_t s);
void launch_resolve_mixed(const LaunchSet& ls, uint32_t display, cudaStream_t s);

// counting-sort photon grid (kernels_grid.cu): scan tiles for a launch's hash slots, and the
// scan of the slots' counts + the scatter of the records, after the photon pass's last store
uint32_t grid_tiles(uint32_t hash_slots);
void launch_grid_sort(const LaunchSet& hash_slots, const LaunchSet& photons, const PhotonGrid& grid, cudaStream_t s);
void launch_gather_fp32(const LaunchSet& ls, uint32_t block, cudaStream_t s);
void launch_resolve_fp32(const LaunchSet& ls, uint32_t display, cudaStream_t s);
void launch_hash_build(const float4* pos, const float4* flux, uint32_t pw, uint32_t ph, uint32_t hash_num,
                       const float bbmin[3], float grid_scale, uint32_t flags, uint32_t* winner, uint32_t* count,
                       cudaStream_t s);
void launch_debug_trace(const DevScene& sc, const float* org, const float* dir, uint32_t n, bool photon, bool cull,
                        int mode, int32_t* tri, float* t, uint32_t* err, cudaStream_t s);
void launch_fpmath(int fn, const float* x, const float* y, float* out, uint32_t n, cudaStream_t s);

}  // namespace sppm_dev

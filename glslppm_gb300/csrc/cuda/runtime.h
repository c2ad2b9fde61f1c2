// Host runtime of the SPPM path: render jobs in device memory and the runner that queues the
// passes of a set of jobs.
//
// A Job owns one scene (traversal layout), camera, progressive state and hashed grid in two
// device arenas.  A Runner owns a stream, a table of job descriptors, the launch tables (job ids
// and prefix sums of each job's pixels, photon slots and hash slots), the shared wavefront ray
// queue and the per-frame CUDA graphs: every stage of a frame is ONE launch over all of its jobs
// (the kernels find an item's job by binary search in the prefix table).  The single-job context
// of sppm.h is a Runner with one job; the batch of sppm_batch.h is a Runner with many.
#pragma once

#include <cstdint>
#include <deque>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "../host/scene_bvh4.h"
#include "../host/scene_internal.h"
#include "device_common.cuh"
#include "sppm.h"

#define SPPM_CK(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return sppm::fail(SPPM_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
                              __FILE__, __LINE__);                                                     \
    } while (0)

namespace sppm_rt {

using namespace sppm_dev;

// bump allocator over one cudaMalloc
struct Arena {
    char* base = nullptr;
    size_t size = 0, used = 0;
    Arena() = default;
    Arena(const Arena&) = delete;
    Arena& operator=(const Arena&) = delete;
    ~Arena() { release(); }
    static size_t align(size_t n) { return (n + 255) & ~size_t(255); }
    void release() {
        if (base) cudaFree(base);
        base = nullptr;
        size = used = 0;
    }
    int reserve(size_t bytes);
    template <class T>
    T* take(size_t count) {
        const size_t b = align(sizeof(T) * count);
        if (used + b > size) return nullptr;
        T* p = reinterpret_cast<T*>(base + used);
        used += b;
        return p;
    }
};

int validate_config(const sppm_config* c);
// state kinds whose device layout differs from what readers get: the mixed-precision statistics
// are double-float pairs on the device and doubles for the reader (converted in place), unless the
// job keeps IEEE doubles (SPPM_FLAG_FP64_STATISTICS); a slot winner equal to the photon count P
// (every photon of the slot clipped) reads back as no winner
void state_to_host_layout(uint32_t kind, void* buf, size_t bytes, uint32_t flags, uint32_t photon_slots);
int launch_check(const char* what);

// the caller's view of a job's frame counters
void fill_frame_info(const JobState& st, sppm_frame_info* fi);

// a scene in the device layout, on the host (CGPURT::CreateTextures, gpurt.cpp:47-552, in the
// traversal layout)
struct Packed {
    std::vector<NodeX> nodes;
    std::vector<float4> isect, shade;
    std::vector<DevMaterial> mats;
    std::vector<float> light_cdf;
    std::vector<int32_t> light_tri;
    std::vector<float2> tri_tex;     // empty when no texture coordinate is below 1e10
    std::vector<int32_t> mat_layer;  // [num_materials]
    std::vector<int32_t> rank;       // [6][num_tris] leaf position of each triangle per ordering
};

// the host-side work of a scene upload -- the traversal layout of the six orderings, the 4-wide
// tree with its emitter marks, the leaf ranks, a copy of the textures, the checkpoint fingerprint
// -- done ahead of time on any thread (sppm_scene_prepare); Job::upload_prepared then allocates
// and copies only
struct PreparedScene {
    Packed pk;
    std::vector<sppm::Node4> nodes4;  // empty when the tree failed or is deeper than the walk's stack
    int bvh4_status = 0;              // build_bvh4's result
    uint32_t bvh4_depth = 0;
    std::vector<uint8_t> textures;
    sppm_scene shape{};               // the source's counts, light area and bounds (no arrays)
    uint64_t fingerprint = 0;
    uint64_t device_bytes = 0;        // of the scene arena
};
int prepare_scene(const sppm_scene* scene, PreparedScene& out);

// a job's seeded random-state tables (RandomizeTextures, glslppm.cpp:77-140: a host-side fill),
// made ahead of time on any thread (sppm_state_prepare); Job::reset then copies them
struct PreparedState {
    std::vector<float> eye, ph;
    uint32_t xs[4] = {0, 0, 0, 0};
    uint32_t npix = 0, P = 0, seed = 0, seed_mode = 0;
    bool matches(const sppm_config& cfg) const;
};
void prepare_state(const sppm_config& cfg, PreparedState& out);

// one render job (scene + camera + progressive state)
struct Job {
    sppm_config cfg{};
    uint32_t W = 0, H = 0, PW = 0, PH = 0, P = 0, npix = 0, hash_num = 0;
    Arena state_mem, scene_mem;
    JobDesc desc{};                // host copy of the device descriptor
    JobDesc* d_desc = nullptr;     // the descriptor's slot in the runner's table
    JobState* d_state = nullptr;
    uint32_t* d_self = nullptr;    // launch tables of this job alone: {slot, 0, npix, 0, P, 0, hash}
    float* d_image = nullptr;
    uint32_t slot = 0;
    bool have_scene = false, have_camera = false;
    float fixed_radius = 0.0f;
    // pinned staging slots for descriptor uploads, so that a camera change is queued without
    // waiting for the frames already queued (slot k is reused once its copy has run)
    JobDesc* stage = nullptr;
    JobDesc* stage_dev = nullptr;  // the slots' address on the device (mapped host memory)
    cudaEvent_t stage_ev[4] = {};
    bool stage_used[4] = {};
    uint32_t stage_next = 0;
    // the last image copy queued on the runner's copy stream (it reads d_image, which the next
    // resolve overwrites)
    cudaEvent_t copy_ev = nullptr;
    bool copy_pending = false;
    Job() = default;
    Job(const Job&) = delete;
    Job& operator=(const Job&) = delete;
    ~Job();
    int64_t start_frame = 0;       // runner frame at which the job's frame 0 is (or was) queued;
                                   // negative for a job resumed with more frames than the runner
    // the runner phase (frame mod interval) at which this job's eye passes fall
    uint32_t eye_phase(uint32_t interval) const {
        const int64_t L = (int64_t)interval;
        return (uint32_t)(((start_frame % L) + L) % L);
    }
    uint64_t scene_bytes_used = 0;
    // fingerprints of the uploaded scene (every input array) and of the camera, recorded in a
    // checkpoint so that it only loads into a job that renders the same thing
    uint64_t scene_fp = 0, camera_fp = 0;

    // device bytes of the state arena for a configuration
    static uint64_t state_bytes(const sppm_config& cfg);
    // device bytes of the scene arena for a scene (mixed precision adds the 4-wide BVH, bounded
    // by the binary node count)
    static uint64_t scene_bytes(const sppm_scene& s, uint32_t precision);

    int init(const sppm_config& cfg, JobDesc* d_desc, uint32_t slot, cudaStream_t s);
    int upload_scene(const sppm_scene* scene, cudaStream_t s);
    int upload_prepared(const PreparedScene& p, cudaStream_t s, const PreparedState* ps = nullptr);
    int set_camera(const sppm_camera* cam, cudaStream_t s);
    int set_camera_desc(const sppm_camera* cam);  // host descriptor only; uploaded by the caller
    int reset(cudaStream_t s, const PreparedState* ps = nullptr);  // ps: tables seeded ahead of time
    int write_desc(cudaStream_t s);
    int stage_desc(const JobDesc** src);  // write_desc in two halves, for uploads of many jobs
    int staged(cudaStream_t s);           // in one launch (launch_copy_descs)
    void* state_ptr(uint32_t kind, size_t* bytes) const;
    int frame_info(sppm_frame_info* fi, cudaStream_t s) const;
    // checkpoint: header + JobState + every state array (flat binary, this build's layout)
    size_t checkpoint_bytes() const;
    int save_checkpoint(void* dst, size_t bytes, cudaStream_t s) const;
    int load_checkpoint(const void* src, size_t bytes, cudaStream_t s, uint32_t* frames_started);
    LaunchSet self_set(const JobDesc* table, uint32_t which) const;  // 0 pixels, 1 photons, 2 hash
    uint64_t bytes() const { return state_mem.size + scene_mem.size; }
};

struct StageEvent {
    int stage;
    cudaEvent_t a, b;
};

// one frame's launches as an instantiated CUDA graph; stages being timed carry event record
// nodes whose events are swapped for pooled ones before every replay
struct FrameGraph {
    cudaGraph_t graph = nullptr;  // kept: the event record nodes below belong to it
    cudaGraphExec_t exec = nullptr;
    uint32_t mask = 0;
    uint32_t kernels = 0;   // kernel nodes (launches per replay)
    bool counting = false;  // captured with the traversal-counting kernels
    bool textured = false;  // captured with the kernel variants that look up textures
    bool fp64 = false;      // captured with the gather variant for IEEE double statistics
    bool wide = false;      // captured with the plain path tracing through the 4-wide BVH
    cudaGraphNode_t ev_a[SPPM_STAGE_COUNT] = {}, ev_b[SPPM_STAGE_COUNT] = {};
    void drop();
};

// queues the frames of a set of jobs on one stream
constexpr uint32_t kDefaultGridCellSplit = 2;

struct Runner {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;             // the eye pass's branch, forked from and joined to stream
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // image copies to host memory run on `copy` beside the passes queued after them; each has a
    // ticket (numbered from 1) whose event marks its end
    cudaStream_t copy = nullptr;
    cudaEvent_t resolved_ev = nullptr;
    // recorded on `copy` after each resolve that runs there (an asynchronous image read): the next
    // frame's eye pass and gather, which overwrite what the resolve reads, wait for it (in a frame
    // graph as external event-wait nodes)
    cudaEvent_t resolve_done = nullptr;
    struct Ticket {
        uint64_t id;
        cudaEvent_t ev;
    };
    std::deque<Ticket> tickets;   // copies whose end has not been observed, oldest first
    std::vector<cudaEvent_t> ticket_pool;
    uint64_t next_ticket = 1;
    Arena info_mem;                 // JobState[max_jobs] gathered by frame_infos
    JobState* info_host = nullptr;  // page-locked copy
    uint32_t precision = SPPM_PRECISION_FP32, flags = 0, eye_interval = 10, max_jobs = 0;
    Arena desc_mem;                // JobDesc[max_jobs]
    JobDesc* d_jobs = nullptr;
    Arena table_mem, queue_mem;    // rebuilt when the set of jobs changes
    RayQueue queue{};
    Arena grid_mem;                // counting-sort photon grid (jobs with SPPM_FLAG_PHOTON_GRID)
    PhotonGrid grid{};
    uint64_t grid_slots_cap = 0, grid_photons_cap = 0;
    uint32_t grid_tiles_cap = 0;
    bool any_grid = false;         // some active job uses the counting-sort photon grid
    // log2 of the grid cells per reference cell along an axis (sppm_tuning.grid_cell_split)
    uint32_t grid_shift() const {
        const uint32_t s = tune.grid_cell_split ? tune.grid_cell_split : kDefaultGridCellSplit;
        return s >= 8 ? 3u : s >= 4 ? 2u : s >= 2 ? 1u : 0u;
    }
    bool any_slot_records = false; // some active mixed job gathers from the slot records
    std::vector<Job*> active;      // launch order
    LaunchSet pix{}, pho{}, hsh{};
    LaunchSet pix_tiles{};         // the pixels in 8x4 tiles, a warp per tile (the grid gather)
    std::vector<LaunchSet> eye_pix;          // per phase (frame mod eye_interval)
    std::vector<const uint32_t*> eye_ids;    // per phase: the job ids of eye_pix
    uint64_t frames = 0;                     // frames queued
    uint64_t kernel_launches = 0;
    uint32_t trace_blocks = 0;
    uint32_t sms = 0, trace_fit = 0;  // SMs; traversal blocks of 128 threads that fit on one SM
    sppm_tuning tune{};               // launch shapes (zero fields: the defaults)
    bool dirty = true;
    // stage timing
    uint32_t timing_mask = 0;  // bit k: time stage k
    bool count_traversal = false;
    bool textured = false;         // some active job's scene has texture coordinates
    bool fp64_stats = false;       // some active job keeps IEEE double statistics
    bool wide_ok = false;          // every active job has the 4-wide BVH (the plain path may use it)
    uint32_t trace_fit4 = 0;       // 4-wide traversal blocks of 128 threads that fit on one SM
    std::vector<StageEvent> pending;
    size_t open_stage[SPPM_STAGE_COUNT] = {0};  // pending entry of each stage's last start
    std::vector<cudaEvent_t> event_pool;
    float stage_ms[SPPM_STAGE_COUNT] = {0};
    uint32_t stage_launches[SPPM_STAGE_COUNT] = {0};
    // frame graphs: one per phase with eye jobs, and one for phases without
    std::vector<FrameGraph> graphs;
    bool capturing = false;
    cudaEvent_t placeholder[2 * SPPM_STAGE_COUNT] = {};

    Runner() = default;
    Runner(const Runner&) = delete;
    Runner& operator=(const Runner&) = delete;
    ~Runner();
    int init(int device, uint32_t precision, uint32_t flags, uint32_t eye_interval, uint32_t max_jobs);
    void drop_graphs();
    int rebuild();                 // launch tables and queue for `active`
    int run(uint32_t n);           // queue n frames of every active job
    int synchronize();             // waits and reports device-side watchdog errors of every job
    int time(uint32_t n, float* ms);
    // launch shapes: checked, then every frame graph is captured again with them (results do not
    // depend on them); get_tuning reports the shapes in effect
    int set_tuning(const sppm_tuning* t);
    void get_tuning(sppm_tuning* t) const;
    // times the next passes under candidate shapes (coordinate descent, each candidate over
    // `cycles` eye-pass cycles after one untimed cycle) and keeps the fastest
    int autotune(uint32_t cycles, sppm_tuning* best, float* ms_per_pass);
    int read_stage_times(float ms[SPPM_STAGE_COUNT], uint32_t launches[SPPM_STAGE_COUNT]);
    int resolve(Job& j, uint32_t kind, cudaStream_t s = nullptr);  // on `stream` by default
    // resolve + copy of the image into host memory without waiting; *ticket names the copy
    int read_image_async(Job& j, uint32_t kind, float* rgb, size_t bytes, uint64_t* ticket);
    // waits for the copy of `ticket` (block) or reports whether it has ended (*done)
    int image_wait(uint64_t ticket, bool block, int* done);
    // the frame counters of several jobs: one gather kernel and one copy
    int frame_infos(Job* const* jobs, uint32_t n, sppm_frame_info* out);
    cudaEvent_t get_event();
    void timed(int stage, bool start, cudaStream_t s = nullptr);

  private:
    void wait_resolve(cudaStream_t s);  // the last asynchronous resolve, before its inputs change
    int enqueue_frame(uint32_t phase);
    int build_graph(uint32_t phase, FrameGraph& g);
    bool phase_has_eye(uint32_t phase) const;
};

}  // namespace sppm_rt

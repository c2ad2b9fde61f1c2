// C ABI of the single-job SPPM context (include/sppm.h) and the stage-level entry points.
//
// A context is a Runner (stream, launch tables, ray queue, frame graphs) holding one Job (scene,
// camera, progressive state).  A frame is queued as the launch sequence of m_display
// (glslppm.cpp:214-536); the scalars the reference reads back between its draws (bounding box,
// photon count) stay on the device.
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"
#include "runtime.h"

using namespace sppm_dev;
using namespace sppm_rt;
using sppm::fail;

struct sppm_ctx {
    Runner rt;
    Job job;
};

extern "C" {

void sppm_config_defaults(sppm_config* c, uint32_t resolution) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->width = c->height = resolution;
    c->photon_width = c->photon_height = resolution;
    c->hash_slots = 0;
    c->max_path_length = 10;
    c->eye_pass_interval = 10;
    c->alpha = 0.7f;
    c->initial_footprint = 2.5f;
    c->radius_rule = SPPM_RADIUS_FOOTPRINT;
    c->radius_fraction = 0.005f;
    c->precision = SPPM_PRECISION_FP32;
    c->seed_mode = SPPM_SEED_XORSHIFT;
    c->seed = 0;
    c->flags = SPPM_FLAG_GL_DEPTH_CLIP;
    c->focal_length = 13.0f;
    c->aperture = 0.0f;
}

int sppm_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int sppm_create(const sppm_config* cfg, int device, sppm_ctx** out) {
    if (!out) return fail(SPPM_ERR_ARG, "null output pointer");
    *out = nullptr;
    int st = validate_config(cfg);
    if (st) return st;
    const int ndev = sppm_device_count();
    if (ndev == 0) return fail(SPPM_ERR_NO_DEVICE, "no CUDA device is visible");
    if (device < 0 || device >= ndev) return fail(SPPM_ERR_ARG, "device %d out of range (%d devices)", device, ndev);
    std::unique_ptr<sppm_ctx> c(new (std::nothrow) sppm_ctx());
    if (!c) return fail(SPPM_ERR_OOM, "host allocation failed");
    if ((st = c->rt.init(device, cfg->precision, cfg->flags, cfg->eye_pass_interval, 1))) return st;
    if ((st = c->job.init(*cfg, c->rt.d_jobs, 0, c->rt.stream))) return st;
    c->job.start_frame = (int64_t)c->rt.frames;
    c->rt.active.push_back(&c->job);
    c->rt.dirty = true;
    *out = c.release();
    return SPPM_OK;
}

int sppm_upload_scene(sppm_ctx* c, const sppm_scene* scene) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaStreamSynchronize(c->rt.stream));
    int st = c->job.upload_scene(scene, c->rt.stream);
    if (st) return st;
    c->job.start_frame = (int64_t)c->rt.frames;
    c->rt.dirty = true;
    return SPPM_OK;
}

int sppm_set_camera(sppm_ctx* c, const sppm_camera* cam) {
    if (!c || !cam) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->rt.device));
    return c->job.set_camera(cam, c->rt.stream);
}

int sppm_reset(sppm_ctx* c) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaStreamSynchronize(c->rt.stream));
    int st = c->job.reset(c->rt.stream);
    if (st) return st;
    c->job.start_frame = (int64_t)c->rt.frames;
    c->rt.dirty = true;
    return SPPM_OK;
}

int sppm_run_passes(sppm_ctx* c, uint32_t n) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    if (!c->job.have_scene || !c->job.have_camera)
        return fail(SPPM_ERR_STATE, "upload a scene and set a camera before running passes");
    return c->rt.run(n);
}

int sppm_synchronize(sppm_ctx* c) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    return c->rt.synchronize();
}

size_t sppm_camera_upload_bytes(void) { return sizeof(JobDesc); }

int sppm_read_image(sppm_ctx* c, uint32_t kind, float* rgb, size_t num_floats) {
    if (!c || !rgb) return fail(SPPM_ERR_ARG, "null argument");
    if (kind > SPPM_IMAGE_DISPLAY) return fail(SPPM_ERR_ARG, "unknown image kind %u", kind);
    if (num_floats != (size_t)c->job.npix * 3)
        return fail(SPPM_ERR_ARG, "image needs %zu floats", (size_t)c->job.npix * 3);
    int st = c->rt.resolve(c->job, kind);
    if (st) return st;
    SPPM_CK(cudaMemcpyAsync(rgb, c->job.d_image, num_floats * 4, cudaMemcpyDeviceToHost, c->rt.stream));
    return c->rt.synchronize();
}

int sppm_read_image_async(sppm_ctx* c, uint32_t kind, float* rgb, size_t num_floats, uint64_t* ticket) {
    if (!c || !rgb || !ticket) return fail(SPPM_ERR_ARG, "null argument");
    if (kind > SPPM_IMAGE_DISPLAY) return fail(SPPM_ERR_ARG, "unknown image kind %u", kind);
    if (num_floats != (size_t)c->job.npix * 3)
        return fail(SPPM_ERR_ARG, "image needs %zu floats", (size_t)c->job.npix * 3);
    return c->rt.read_image_async(c->job, kind, rgb, num_floats * 4, ticket);
}

int sppm_image_wait(sppm_ctx* c, uint64_t ticket) {
    if (!c) return fail(SPPM_ERR_ARG, "null argument");
    return c->rt.image_wait(ticket, true, nullptr);
}

int sppm_image_query(sppm_ctx* c, uint64_t ticket, int* done) {
    if (!c || !done) return fail(SPPM_ERR_ARG, "null argument");
    return c->rt.image_wait(ticket, false, done);
}

size_t sppm_state_bytes(const sppm_ctx* c, uint32_t kind) {
    if (!c) return 0;
    size_t b = 0;
    return c->job.state_ptr(kind, &b) ? b : 0;
}

int sppm_read_state(sppm_ctx* c, uint32_t kind, void* dst, size_t bytes) {
    if (!c || !dst) return fail(SPPM_ERR_ARG, "null argument");
    size_t need = 0;
    void* src = c->job.state_ptr(kind, &need);
    if (!src) return fail(SPPM_ERR_ARG, "state kind %u is not kept by this context", kind);
    if (bytes != need) return fail(SPPM_ERR_ARG, "state kind %u has %zu bytes, %zu requested", kind, need, bytes);
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->rt.stream));
    const int st = c->rt.synchronize();
    if (st == SPPM_OK) state_to_host_layout(kind, dst, bytes, c->job.cfg.flags, c->job.P);
    return st;
}

size_t sppm_checkpoint_bytes(const sppm_ctx* c) { return c ? c->job.checkpoint_bytes() : 0; }

int sppm_save_checkpoint(sppm_ctx* c, void* dst, size_t bytes) {
    if (!c || !dst) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaStreamSynchronize(c->rt.stream));
    return c->job.save_checkpoint(dst, bytes, c->rt.stream);
}

int sppm_load_checkpoint(sppm_ctx* c, const void* src, size_t bytes) {
    if (!c || !src) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->rt.device));
    uint32_t frames = 0;
    int st = c->job.load_checkpoint(src, bytes, c->rt.stream, &frames);
    if (st) return st;
    // the job's next frame is frame `frames`: its eye-pass phase follows
    c->job.start_frame = (int64_t)c->rt.frames - (int64_t)frames;
    c->rt.dirty = true;
    return SPPM_OK;
}

int sppm_get_frame_info(sppm_ctx* c, sppm_frame_info* fi) {
    if (!c || !fi) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->rt.device));
    int st = c->job.frame_info(fi, c->rt.stream);
    if (st) return st;
    fi->kernel_launches = c->rt.kernel_launches;
    return SPPM_OK;
}

int sppm_enable_traversal_counters(sppm_ctx* c, int enable) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    c->rt.count_traversal = enable != 0;
    return SPPM_OK;
}

int sppm_enable_stage_timing(sppm_ctx* c, int enable) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    c->rt.timing_mask = enable ? (1u << SPPM_STAGE_COUNT) - 1u : 0u;
    return SPPM_OK;
}

int sppm_set_stage_timing_mask(sppm_ctx* c, uint32_t mask) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    c->rt.timing_mask = mask & ((1u << SPPM_STAGE_COUNT) - 1u);
    return SPPM_OK;
}

int sppm_read_stage_times(sppm_ctx* c, float ms[SPPM_STAGE_COUNT], uint32_t launches[SPPM_STAGE_COUNT]) {
    if (!c || !ms || !launches) return fail(SPPM_ERR_ARG, "null argument");
    return c->rt.read_stage_times(ms, launches);
}

int sppm_time_passes(sppm_ctx* c, uint32_t n, float* ms) {
    if (!c || !ms) return fail(SPPM_ERR_ARG, "null argument");
    if (!c->job.have_scene || !c->job.have_camera)
        return fail(SPPM_ERR_STATE, "upload a scene and set a camera before running passes");
    return c->rt.time(n, ms);
}

int sppm_set_tuning(sppm_ctx* c, const sppm_tuning* t) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    return c->rt.set_tuning(t);
}

int sppm_get_tuning(sppm_ctx* c, sppm_tuning* t) {
    if (!c || !t) return fail(SPPM_ERR_ARG, "null argument");
    c->rt.get_tuning(t);
    return SPPM_OK;
}

int sppm_autotune(sppm_ctx* c, uint32_t cycles, sppm_tuning* best, float* ms_per_pass) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    if (!c->job.have_scene || !c->job.have_camera)
        return fail(SPPM_ERR_STATE, "upload a scene and set a camera before tuning");
    return c->rt.autotune(cycles, best, ms_per_pass);
}

int sppm_tune_hash_slots(const sppm_config* cfg, const sppm_scene* scene, const sppm_camera* cam, int device,
                         uint32_t passes, uint32_t* hash_slots, float ms_out[3]) {
    if (!cfg || !scene || !cam || !hash_slots || !passes) return fail(SPPM_ERR_ARG, "null argument or zero passes");
    int st = validate_config(cfg);
    if (st) return st;
    const uint64_t P = (uint64_t)cfg->photon_width * cfg->photon_height;
    float best = 0.0f;
    for (uint32_t k = 0; k < 3; k++) {
        const uint64_t slots = P << k;
        if (slots > (1ull << 28)) {
            if (ms_out) ms_out[k] = -1.0f;  // beyond the largest table a configuration may ask for
            continue;
        }
        sppm_config c = *cfg;
        c.hash_slots = (uint32_t)slots;
        sppm_ctx* ctx = nullptr;
        float ms = 0.0f;
        if ((st = sppm_create(&c, device, &ctx)) || (st = sppm_upload_scene(ctx, scene)) ||
            (st = sppm_set_camera(ctx, cam)) || (st = sppm_run_passes(ctx, passes)) ||
            (st = sppm_time_passes(ctx, passes, &ms))) {
            sppm_destroy(ctx);
            return st;
        }
        sppm_destroy(ctx);
        if (ms_out) ms_out[k] = ms / (float)passes;
        if (k == 0 || ms < 0.99f * best) {
            best = ms;
            *hash_slots = (uint32_t)slots;
        }
    }
    return SPPM_OK;
}

void sppm_destroy(sppm_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->rt.device);
    if (c->rt.stream) cudaStreamSynchronize(c->rt.stream);
    delete c;
}

int sppm_hash_build(const float* d_pos, const float* d_flux, uint32_t pw, uint32_t ph, uint32_t hash_slots,
                    const float bbox_min[3], float grid_scale, uint32_t flags, uint32_t* d_winner, uint32_t* d_count,
                    void* stream) {
    if (!d_pos || !d_flux || !bbox_min || !d_winner || !d_count) return fail(SPPM_ERR_ARG, "null argument");
    if (pw == 0 || ph == 0 || hash_slots == 0) return fail(SPPM_ERR_ARG, "empty photon buffer or hash table");
    if ((uint64_t)pw * ph > (1u << 30)) return fail(SPPM_ERR_ARG, "photon buffer too large");
    if (!(grid_scale > 0.0f)) return fail(SPPM_ERR_ARG, "grid_scale must be positive");
    if ((reinterpret_cast<uintptr_t>(d_pos) | reinterpret_cast<uintptr_t>(d_flux)) & 15)
        return fail(SPPM_ERR_ARG, "pos/flux must be 16-byte aligned float4 arrays");
    launch_hash_build(reinterpret_cast<const float4*>(d_pos), reinterpret_cast<const float4*>(d_flux), pw, ph,
                      hash_slots, bbox_min, grid_scale, flags, d_winner, d_count, (cudaStream_t)stream);
    return launch_check("hash build");
}

int sppm_debug_fpmath(int fn, const float* x, const float* y, float* out, size_t n) {
    if (!x || !out || (fn == 2 && !y)) return fail(SPPM_ERR_ARG, "null argument");
    if (n == 0) return SPPM_OK;
    if (n > (1u << 28)) return fail(SPPM_ERR_ARG, "n too large");
    if (sppm_device_count() == 0) return fail(SPPM_ERR_NO_DEVICE, "no CUDA device is visible");
    float *dx = nullptr, *dy = nullptr, *dout = nullptr;
    SPPM_CK(cudaMalloc(&dx, n * 4));
    SPPM_CK(cudaMalloc(&dy, n * 4));
    SPPM_CK(cudaMalloc(&dout, n * 4));
    cudaMemcpy(dx, x, n * 4, cudaMemcpyHostToDevice);
    if (y) cudaMemcpy(dy, y, n * 4, cudaMemcpyHostToDevice);
    launch_fpmath(fn, dx, dy, dout, (uint32_t)n, 0);
    cudaError_t e = cudaMemcpy(out, dout, n * 4, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dout);
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "fpmath kernel failed: %s", cudaGetErrorString(e));
    return SPPM_OK;
}

int sppm_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(SPPM_ERR_ARG, "null argument");
    *ptr = nullptr;
    if (bytes == 0) return SPPM_OK;
    if (sppm_device_count() == 0) return fail(SPPM_ERR_NO_DEVICE, "no CUDA device is visible");
    const cudaError_t e = cudaMallocHost(ptr, bytes);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(e == cudaErrorMemoryAllocation ? SPPM_ERR_OOM : SPPM_ERR_CUDA, "cudaMallocHost(%zu) failed: %s",
                    bytes, cudaGetErrorString(e));
    }
    return SPPM_OK;
}

void sppm_host_free(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
}

int sppm_debug_photon_rays(sppm_ctx* c, float* org, float* dir, uint32_t* photon, size_t capacity, size_t* count) {
    if (!c || !count) return fail(SPPM_ERR_ARG, "null argument");
    if (c->rt.flags & SPPM_FLAG_FUSED_PHOTON)
        return fail(SPPM_ERR_STATE, "the fused photon kernel keeps no ray queue");
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaStreamSynchronize(c->rt.stream));
    const RayQueue& q = c->rt.queue;
    uint32_t n = 0;
    if (q.counters) SPPM_CK(cudaMemcpy(&n, q.counters, 4, cudaMemcpyDeviceToHost));
    *count = n;
    if (!org && !dir && !photon) return SPPM_OK;  // size query
    if (!org || !dir || !photon) return fail(SPPM_ERR_ARG, "null argument");
    if (capacity < n) return fail(SPPM_ERR_ARG, "the last pass traced %u photon rays; capacity %zu", n, capacity);
    std::vector<float4> o(n), d(n);
    if (n) {
        SPPM_CK(cudaMemcpy(o.data(), q.org, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost));
        SPPM_CK(cudaMemcpy(d.data(), q.dir, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost));
    }
    for (uint32_t i = 0; i < n; i++) {
        org[3 * i] = o[i].x, org[3 * i + 1] = o[i].y, org[3 * i + 2] = o[i].z;
        dir[3 * i] = d[i].x, dir[3 * i + 1] = d[i].y, dir[3 * i + 2] = d[i].z;
        uint32_t g;
        memcpy(&g, &o[i].w, 4);
        photon[i] = g;
    }
    return SPPM_OK;
}

int sppm_debug_photon_grid(sppm_ctx* c, uint32_t* offsets, size_t offsets_capacity, uint32_t* records,
                           size_t records_capacity, uint32_t* num_records) {
    if (!c || !num_records) return fail(SPPM_ERR_ARG, "null argument");
    if (!(c->job.cfg.flags & SPPM_FLAG_PHOTON_GRID))
        return fail(SPPM_ERR_STATE, "the context was created without SPPM_FLAG_PHOTON_GRID");
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaStreamSynchronize(c->rt.stream));
    const PhotonGrid& g = c->rt.grid;
    if (!g.ofs || c->rt.frames == 0) return fail(SPPM_ERR_STATE, "no pass has run yet");
    const uint32_t hn = c->job.hash_num;
    uint32_t n = 0;
    SPPM_CK(cudaMemcpy(&n, g.ofs + hn, 4, cudaMemcpyDeviceToHost));
    *num_records = n;
    if (!offsets && !records) return SPPM_OK;  // size query
    if (!offsets || !records) return fail(SPPM_ERR_ARG, "null argument");
    if (offsets_capacity < (size_t)hn + 1 || records_capacity < (size_t)n * 4)
        return fail(SPPM_ERR_ARG, "the grid holds %u slots and %u records: capacities %zu and %zu words", hn, n,
                    offsets_capacity, records_capacity);
    SPPM_CK(cudaMemcpy(offsets, g.ofs, ((size_t)hn + 1) * 4, cudaMemcpyDeviceToHost));
    if (n) SPPM_CK(cudaMemcpy(records, g.rec, (size_t)n * 16, cudaMemcpyDeviceToHost));
    return SPPM_OK;
}

int sppm_debug_ray_bins(sppm_ctx* c, uint32_t* rank, uint64_t* cost, size_t capacity, uint32_t* num_bins) {
    if (!c || !num_bins) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaStreamSynchronize(c->rt.stream));
    const RayQueue& q = c->rt.queue;
    if (!q.bin_rank || !q.bin_cost) return fail(SPPM_ERR_STATE, "no ray bins: created unbinned, or no pass has run");
    *num_bins = kRayBins;
    if (!rank && !cost) return SPPM_OK;  // size query
    if (!rank || !cost) return fail(SPPM_ERR_ARG, "null argument");
    if (capacity < kRayBins) return fail(SPPM_ERR_ARG, "capacity %zu < %u bins", capacity, kRayBins);
    SPPM_CK(cudaMemcpy(rank, q.bin_rank, (size_t)kRayBins * 4, cudaMemcpyDeviceToHost));
    SPPM_CK(cudaMemcpy(cost, q.bin_cost, (size_t)kRayBins * 8, cudaMemcpyDeviceToHost));
    return SPPM_OK;
}

int sppm_debug_trace(sppm_ctx* c, const float* org, const float* dir, size_t n, int photon, int cull, int mode,
                     int32_t* tri, float* t) {
    if (!c || !org || !dir || !tri || !t) return fail(SPPM_ERR_ARG, "null argument");
    if (!c->job.have_scene) return fail(SPPM_ERR_STATE, "upload a scene first");
    if (mode < 0 || mode > 3)
        return fail(SPPM_ERR_ARG,
                    "mode must be 0 (thread per ray), 1 (warp per ray), 2 (block per ray) or 3 (4-wide quantised)");
    if (mode == 3 && !c->job.desc.scene.nodes4)
        return fail(SPPM_ERR_STATE, "mode 3 traces the mixed-precision 4-wide BVH: create the context with "
                                    "SPPM_PRECISION_MIXED");
    if (n == 0) return SPPM_OK;
    if (n > (1u << 26)) return fail(SPPM_ERR_ARG, "n too large");
    SPPM_CK(cudaSetDevice(c->rt.device));
    SPPM_CK(cudaStreamSynchronize(c->rt.stream));
    float *d_org = nullptr, *d_dir = nullptr, *d_t = nullptr;
    int32_t* d_tri = nullptr;
    uint32_t* d_err = nullptr;
    cudaError_t e = cudaMalloc(&d_org, n * 12);
    if (e == cudaSuccess) e = cudaMalloc(&d_dir, n * 12);
    if (e == cudaSuccess) e = cudaMalloc(&d_t, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_tri, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_err, 4);
    if (e == cudaSuccess) e = cudaMemcpy(d_org, org, n * 12, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_dir, dir, n * 12, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_err, 0, 4);
    uint32_t err = 0;
    if (e == cudaSuccess) {
        launch_debug_trace(c->job.desc.scene, d_org, d_dir, (uint32_t)n, photon != 0, cull != 0, mode, d_tri, d_t,
                           d_err, c->rt.stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->rt.stream);
    if (e == cudaSuccess) e = cudaMemcpy(tri, d_tri, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(t, d_t, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&err, d_err, 4, cudaMemcpyDeviceToHost);
    cudaFree(d_org);
    cudaFree(d_dir);
    cudaFree(d_t);
    cudaFree(d_tri);
    cudaFree(d_err);
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "debug trace failed: %s", cudaGetErrorString(e));
    if (err) return fail(SPPM_ERR_WATCHDOG, "BVH traversal exceeded its step bound");
    return SPPM_OK;
}

}  // extern "C"

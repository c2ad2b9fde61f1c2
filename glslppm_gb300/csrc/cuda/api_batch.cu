// C ABI of the batched SPPM path (include/sppm_batch.h): a Runner holding many Jobs.
#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"
#include "runtime.h"
#include "sppm_batch.h"

using namespace sppm_dev;
using namespace sppm_rt;
using sppm::fail;

struct sppm_prepared_scene {
    PreparedScene p;
};

struct sppm_prepared_state {
    PreparedState p;
};

struct sppm_batch {
    Runner rt;
    sppm_batch_config cfg{};
    std::vector<std::unique_ptr<Job>> slots;  // [max_jobs]; null = free
    uint64_t budget = 0;
};

namespace {

// ray queue bytes per photon slot: org, dir, hit (3 x 16), set-aside list (4), binning key (8),
// permutation (4), tail-walk list (4) and state (16)
constexpr uint64_t kQueueBytesPerSlot = 3 * 16 + 4 + 8 + 4 + 4 + 16;

Job* job_of(const sppm_batch* b, uint32_t id) {
    if (!b || id >= b->slots.size()) return nullptr;
    return b->slots[id].get();
}

uint64_t used_bytes(const sppm_batch* b) {
    uint64_t u = b->rt.desc_mem.size + b->rt.table_mem.size + b->rt.queue_mem.size;
    for (const auto& j : b->slots)
        if (j) u += j->bytes();
    return u;
}

uint64_t queued_slots(const sppm_batch* b) {
    uint64_t p = 0;
    for (const auto& j : b->slots)
        if (j) p += j->P;
    return p;
}

}  // namespace

namespace {

// the bytes a job holds besides its scene arena: state, its share of the ray queue and, with the
// photon grid, of the launch's grid (a 16-byte record per photon slot, an offset per hash slot)
uint64_t job_bytes_beside_scene(const sppm_config& cfg) {
    const uint64_t P = (uint64_t)cfg.photon_width * cfg.photon_height;
    uint64_t b = Job::state_bytes(cfg) + kQueueBytesPerSlot * P;
    if (cfg.flags & SPPM_FLAG_PHOTON_GRID) b += 16 * P + 4 * (uint64_t)(cfg.hash_slots ? cfg.hash_slots : P);
    return b;
}

int check_job(const sppm_batch* b, const sppm_config* cfg) {
    int st = validate_config(cfg);
    if (st) return st;
    if (cfg->precision != b->cfg.precision)
        return fail(SPPM_ERR_ARG, "job precision %u differs from the batch's %u", cfg->precision, b->cfg.precision);
    const uint32_t interval = cfg->eye_pass_interval ? cfg->eye_pass_interval : 1u;
    if (interval != b->cfg.eye_pass_interval)
        return fail(SPPM_ERR_ARG, "job eye_pass_interval %u differs from the batch's %u", interval,
                    b->cfg.eye_pass_interval);
    return SPPM_OK;
}

// admits a job of `need` device bytes; upload(job) sends its scene
template <class Upload>
int add_job(sppm_batch* b, const sppm_config* cfg, const sppm_camera* cam, uint64_t need, Upload upload,
            uint32_t* job) {
    uint32_t id = 0;
    while (id < b->slots.size() && b->slots[id]) id++;
    if (id == b->slots.size()) return fail(SPPM_ERR_STATE, "every one of the %u job slots is taken", (uint32_t)id);
    const uint64_t used = used_bytes(b);
    if (used + need > b->budget)
        return fail(SPPM_ERR_OOM, "admission: job needs %llu bytes, %llu of the %llu-byte budget are in use",
                    (unsigned long long)need, (unsigned long long)used, (unsigned long long)b->budget);
    SPPM_CK(cudaSetDevice(b->rt.device));
    SPPM_CK(cudaStreamSynchronize(b->rt.stream));
    std::unique_ptr<Job> j(new (std::nothrow) Job());
    if (!j) return fail(SPPM_ERR_OOM, "host allocation failed");
    int st;
    if ((st = j->init(*cfg, b->rt.d_jobs + id, id, b->rt.stream))) return st;
    if ((st = upload(*j))) return st;
    if ((st = j->set_camera(cam, b->rt.stream))) return st;
    j->start_frame = (int64_t)b->rt.frames;
    b->rt.active.push_back(j.get());
    b->slots[id] = std::move(j);
    b->rt.dirty = true;
    *job = id;
    return SPPM_OK;
}

}  // namespace

extern "C" {

void sppm_batch_config_defaults(sppm_batch_config* c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->precision = SPPM_PRECISION_FP32;
    c->flags = 0;
    c->eye_pass_interval = 10;
    c->max_jobs = 256;
    c->memory_budget = 0;
}

int sppm_batch_create(const sppm_batch_config* cfg, int device, sppm_batch** out) {
    if (!cfg || !out) return fail(SPPM_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->precision != SPPM_PRECISION_FP32 && cfg->precision != SPPM_PRECISION_MIXED)
        return fail(SPPM_ERR_ARG, "unknown precision %u", cfg->precision);
    if (cfg->max_jobs == 0 || cfg->max_jobs > 65536) return fail(SPPM_ERR_ARG, "max_jobs must be 1..65536");
    if (cfg->eye_pass_interval > 4096) return fail(SPPM_ERR_ARG, "eye_pass_interval must be at most 4096");
    const int ndev = sppm_device_count();
    if (ndev == 0) return fail(SPPM_ERR_NO_DEVICE, "no CUDA device is visible");
    if (device < 0 || device >= ndev) return fail(SPPM_ERR_ARG, "device %d out of range (%d devices)", device, ndev);
    std::unique_ptr<sppm_batch> b(new (std::nothrow) sppm_batch());
    if (!b) return fail(SPPM_ERR_OOM, "host allocation failed");
    b->cfg = *cfg;
    const uint32_t interval = cfg->eye_pass_interval ? cfg->eye_pass_interval : 1u;
    b->cfg.eye_pass_interval = interval;
    int st = b->rt.init(device, cfg->precision, cfg->flags, interval, cfg->max_jobs);
    if (st) return st;
    b->slots.resize(cfg->max_jobs);
    b->budget = cfg->memory_budget;
    if (b->budget == 0) {
        size_t free_b = 0, total_b = 0;
        SPPM_CK(cudaMemGetInfo(&free_b, &total_b));
        b->budget = (uint64_t)((double)free_b * 0.9);
    }
    *out = b.release();
    return SPPM_OK;
}

void sppm_batch_destroy(sppm_batch* b) {
    if (!b) return;
    cudaSetDevice(b->rt.device);
    if (b->rt.stream) cudaStreamSynchronize(b->rt.stream);
    b->rt.active.clear();
    b->slots.clear();
    delete b;
}

int sppm_batch_job_bytes(const sppm_batch* b, const sppm_config* cfg, const sppm_scene* scene, uint64_t* bytes) {
    if (!b || !cfg || !scene || !bytes) return fail(SPPM_ERR_ARG, "null argument");
    int st = validate_config(cfg);
    if (st) return st;
    *bytes = job_bytes_beside_scene(*cfg) + Job::scene_bytes(*scene, cfg->precision);
    return SPPM_OK;
}

int sppm_batch_job_bytes_prepared(const sppm_batch* b, const sppm_config* cfg, const sppm_prepared_scene* scene,
                                  uint64_t* bytes) {
    if (!b || !cfg || !scene || !bytes) return fail(SPPM_ERR_ARG, "null argument");
    int st = validate_config(cfg);
    if (st) return st;
    *bytes = job_bytes_beside_scene(*cfg) + scene->p.device_bytes;
    return SPPM_OK;
}

int sppm_batch_add_job(sppm_batch* b, const sppm_config* cfg, const sppm_scene* scene, const sppm_camera* cam,
                       uint32_t* job) {
    if (!b || !cfg || !scene || !cam || !job) return fail(SPPM_ERR_ARG, "null argument");
    int st = check_job(b, cfg);
    if (st) return st;
    uint64_t need = 0;
    if ((st = sppm_batch_job_bytes(b, cfg, scene, &need))) return st;
    return add_job(b, cfg, cam, need, [&](Job& j) { return j.upload_scene(scene, b->rt.stream); }, job);
}

int sppm_scene_prepare(const sppm_scene* scene, sppm_prepared_scene** out) {
    if (!scene || !out) return fail(SPPM_ERR_ARG, "null argument");
    *out = nullptr;
    std::unique_ptr<sppm_prepared_scene> p(new (std::nothrow) sppm_prepared_scene());
    if (!p) return fail(SPPM_ERR_OOM, "host allocation failed");
    try {
        const int st = prepare_scene(scene, p->p);
        if (st) return st;
    } catch (const std::bad_alloc&) {
        return fail(SPPM_ERR_OOM, "host allocation failed (scene preparation)");
    }
    *out = p.release();
    return SPPM_OK;
}

void sppm_scene_prepared_destroy(sppm_prepared_scene* scene) { delete scene; }

int sppm_state_prepare(const sppm_config* cfg, sppm_prepared_state** out) {
    if (!cfg || !out) return fail(SPPM_ERR_ARG, "null argument");
    *out = nullptr;
    int st = validate_config(cfg);
    if (st) return st;
    std::unique_ptr<sppm_prepared_state> p(new (std::nothrow) sppm_prepared_state());
    if (!p) return fail(SPPM_ERR_OOM, "host allocation failed");
    try {
        prepare_state(*cfg, p->p);
    } catch (const std::bad_alloc&) {
        return fail(SPPM_ERR_OOM, "host allocation failed (random-state tables)");
    }
    *out = p.release();
    return SPPM_OK;
}

void sppm_state_prepared_destroy(sppm_prepared_state* state) { delete state; }

int sppm_batch_add_job_prepared(sppm_batch* b, const sppm_config* cfg, const sppm_prepared_scene* scene,
                                const sppm_prepared_state* state, const sppm_camera* cam, uint32_t* job) {
    if (!b || !cfg || !scene || !cam || !job) return fail(SPPM_ERR_ARG, "null argument");
    int st = check_job(b, cfg);
    if (st) return st;
    if (state && !state->p.matches(*cfg)) return fail(SPPM_ERR_ARG, "the prepared state is of another configuration");
    uint64_t need = 0;
    if ((st = sppm_batch_job_bytes_prepared(b, cfg, scene, &need))) return st;
    return add_job(
        b, cfg, cam, need,
        [&](Job& j) { return j.upload_prepared(scene->p, b->rt.stream, state ? &state->p : nullptr); }, job);
}

int sppm_batch_remove_job(sppm_batch* b, uint32_t id) {
    Job* j = job_of(b, id);
    if (!j) return fail(SPPM_ERR_ARG, "no job %u", id);
    SPPM_CK(cudaSetDevice(b->rt.device));
    SPPM_CK(cudaStreamSynchronize(b->rt.stream));
    auto& a = b->rt.active;
    a.erase(std::remove(a.begin(), a.end(), j), a.end());
    b->slots[id].reset();
    b->rt.dirty = true;
    return SPPM_OK;
}

int sppm_batch_reset_job(sppm_batch* b, uint32_t id) {
    Job* j = job_of(b, id);
    if (!j) return fail(SPPM_ERR_ARG, "no job %u", id);
    SPPM_CK(cudaSetDevice(b->rt.device));
    SPPM_CK(cudaStreamSynchronize(b->rt.stream));
    int st = j->reset(b->rt.stream);
    if (st) return st;
    j->start_frame = (int64_t)b->rt.frames;
    b->rt.dirty = true;
    return SPPM_OK;
}

int sppm_batch_set_camera(sppm_batch* b, uint32_t id, const sppm_camera* cam) {
    Job* j = job_of(b, id);
    if (!j || !cam) return fail(SPPM_ERR_ARG, "no job %u or null camera", id);
    SPPM_CK(cudaSetDevice(b->rt.device));
    return j->set_camera(cam, b->rt.stream);
}

int sppm_batch_set_cameras(sppm_batch* b, uint32_t n, const uint32_t* ids, const sppm_camera* cams) {
    if (!b || (n && (!ids || !cams))) return fail(SPPM_ERR_ARG, "null batch, job list or camera list");
    std::vector<Job*> js(n);
    for (uint32_t i = 0; i < n; i++) {
        js[i] = job_of(b, ids[i]);
        if (!js[i]) return fail(SPPM_ERR_ARG, "no job %u", ids[i]);
        for (uint32_t p = 0; p < i; p++)
            if (js[p] == js[i]) return fail(SPPM_ERR_ARG, "job %u listed twice", ids[i]);
    }
    SPPM_CK(cudaSetDevice(b->rt.device));
    int st = SPPM_OK;
    for (uint32_t i0 = 0; i0 < n; i0 += kDescCopyMax) {
        const uint32_t m = std::min(n - i0, kDescCopyMax);
        DescCopy list;
        list.n = m;
        for (uint32_t i = 0; i < m; i++) {
            Job* j = js[i0 + i];
            j->set_camera_desc(&cams[i0 + i]);
            if ((st = j->stage_desc(&list.src[i]))) return st;
            list.dst[i] = j->d_desc;
        }
        launch_copy_descs(list, b->rt.stream);
        SPPM_CK(cudaGetLastError());
        for (uint32_t i = 0; i < m; i++)
            if ((st = js[i0 + i]->staged(b->rt.stream))) return st;
    }
    return SPPM_OK;
}

int sppm_batch_run_passes(sppm_batch* b, uint32_t n) {
    if (!b) return fail(SPPM_ERR_ARG, "null batch");
    return b->rt.run(n);
}

int sppm_batch_set_tuning(sppm_batch* b, const sppm_tuning* t) {
    if (!b) return fail(SPPM_ERR_ARG, "null batch");
    return b->rt.set_tuning(t);
}

int sppm_batch_get_tuning(sppm_batch* b, sppm_tuning* t) {
    if (!b || !t) return fail(SPPM_ERR_ARG, "null argument");
    b->rt.get_tuning(t);
    return SPPM_OK;
}

int sppm_batch_autotune(sppm_batch* b, uint32_t cycles, sppm_tuning* best, float* ms_per_pass) {
    if (!b) return fail(SPPM_ERR_ARG, "null batch");
    return b->rt.autotune(cycles, best, ms_per_pass);
}

int sppm_batch_time_passes(sppm_batch* b, uint32_t n, float* ms) {
    if (!b || !ms) return fail(SPPM_ERR_ARG, "null argument");
    return b->rt.time(n, ms);
}

int sppm_batch_synchronize(sppm_batch* b) {
    if (!b) return fail(SPPM_ERR_ARG, "null batch");
    return b->rt.synchronize();
}

int sppm_batch_read_image(sppm_batch* b, uint32_t id, uint32_t kind, float* rgb, size_t num_floats) {
    Job* j = job_of(b, id);
    if (!j || !rgb) return fail(SPPM_ERR_ARG, "no job %u or null buffer", id);
    if (kind > SPPM_IMAGE_DISPLAY) return fail(SPPM_ERR_ARG, "unknown image kind %u", kind);
    if (num_floats != (size_t)j->npix * 3) return fail(SPPM_ERR_ARG, "image needs %zu floats", (size_t)j->npix * 3);
    int st = b->rt.resolve(*j, kind);
    if (st) return st;
    SPPM_CK(cudaMemcpyAsync(rgb, j->d_image, num_floats * 4, cudaMemcpyDeviceToHost, b->rt.stream));
    return b->rt.synchronize();
}

int sppm_batch_read_image_async(sppm_batch* b, uint32_t id, uint32_t kind, float* rgb, size_t num_floats,
                                uint64_t* ticket) {
    Job* j = job_of(b, id);
    if (!j || !rgb || !ticket) return fail(SPPM_ERR_ARG, "no job %u or null argument", id);
    if (kind > SPPM_IMAGE_DISPLAY) return fail(SPPM_ERR_ARG, "unknown image kind %u", kind);
    if (num_floats != (size_t)j->npix * 3) return fail(SPPM_ERR_ARG, "image needs %zu floats", (size_t)j->npix * 3);
    return b->rt.read_image_async(*j, kind, rgb, num_floats * 4, ticket);
}

int sppm_batch_image_wait(sppm_batch* b, uint64_t ticket) {
    if (!b) return fail(SPPM_ERR_ARG, "null argument");
    return b->rt.image_wait(ticket, true, nullptr);
}

int sppm_batch_image_query(sppm_batch* b, uint64_t ticket, int* done) {
    if (!b || !done) return fail(SPPM_ERR_ARG, "null argument");
    return b->rt.image_wait(ticket, false, done);
}

size_t sppm_batch_state_bytes(const sppm_batch* b, uint32_t id, uint32_t kind) {
    const Job* j = job_of(b, id);
    if (!j) return 0;
    size_t n = 0;
    return j->state_ptr(kind, &n) ? n : 0;
}

int sppm_batch_read_state(sppm_batch* b, uint32_t id, uint32_t kind, void* dst, size_t bytes) {
    Job* j = job_of(b, id);
    if (!j || !dst) return fail(SPPM_ERR_ARG, "no job %u or null buffer", id);
    size_t need = 0;
    void* src = j->state_ptr(kind, &need);
    if (!src) return fail(SPPM_ERR_ARG, "state kind %u is not kept by this job", kind);
    if (bytes != need) return fail(SPPM_ERR_ARG, "state kind %u has %zu bytes, %zu requested", kind, need, bytes);
    SPPM_CK(cudaSetDevice(b->rt.device));
    SPPM_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, b->rt.stream));
    const int st = b->rt.synchronize();
    if (st == SPPM_OK) state_to_host_layout(kind, dst, bytes, j->cfg.flags, j->P);
    return st;
}

size_t sppm_batch_checkpoint_bytes(const sppm_batch* b, uint32_t id) {
    const Job* j = job_of(b, id);
    return j ? j->checkpoint_bytes() : 0;
}

int sppm_batch_save_checkpoint(sppm_batch* b, uint32_t id, void* dst, size_t bytes) {
    Job* j = job_of(b, id);
    if (!j || !dst) return fail(SPPM_ERR_ARG, "no job %u or null buffer", id);
    SPPM_CK(cudaSetDevice(b->rt.device));
    SPPM_CK(cudaStreamSynchronize(b->rt.stream));
    return j->save_checkpoint(dst, bytes, b->rt.stream);
}

int sppm_batch_load_checkpoint(sppm_batch* b, uint32_t id, const void* src, size_t bytes) {
    Job* j = job_of(b, id);
    if (!j || !src) return fail(SPPM_ERR_ARG, "no job %u or null buffer", id);
    SPPM_CK(cudaSetDevice(b->rt.device));
    uint32_t frames = 0;
    int st = j->load_checkpoint(src, bytes, b->rt.stream, &frames);
    if (st) return st;
    j->start_frame = (int64_t)b->rt.frames - (int64_t)frames;
    b->rt.dirty = true;
    return SPPM_OK;
}

int sppm_batch_get_frame_info(sppm_batch* b, uint32_t id, sppm_frame_info* fi) {
    Job* j = job_of(b, id);
    if (!j || !fi) return fail(SPPM_ERR_ARG, "no job %u or null output", id);
    SPPM_CK(cudaSetDevice(b->rt.device));
    int st = j->frame_info(fi, b->rt.stream);
    if (st) return st;
    fi->kernel_launches = b->rt.kernel_launches;
    return SPPM_OK;
}

int sppm_batch_get_frame_infos(sppm_batch* b, const uint32_t* ids, uint32_t n, sppm_frame_info* fi) {
    if (!b || (n && (!ids || !fi))) return fail(SPPM_ERR_ARG, "null argument");
    std::vector<Job*> jobs(n);
    for (uint32_t k = 0; k < n; k++) {
        jobs[k] = job_of(b, ids[k]);
        if (!jobs[k]) return fail(SPPM_ERR_ARG, "no job %u", ids[k]);
    }
    return b->rt.frame_infos(jobs.data(), n, fi);
}

size_t sppm_batch_frame_record_bytes(void) { return sizeof(JobState); }

int sppm_batch_get_info(sppm_batch* b, sppm_batch_info* info) {
    if (!b || !info) return fail(SPPM_ERR_ARG, "null argument");
    memset(info, 0, sizeof(*info));
    info->num_jobs = (uint32_t)b->rt.active.size();
    info->max_jobs = (uint32_t)b->slots.size();
    info->bytes_used = used_bytes(b);
    info->memory_budget = b->budget;
    info->frames = b->rt.frames;
    info->kernel_launches = b->rt.kernel_launches;
    info->photon_slots = queued_slots(b);
    for (const Job* j : b->rt.active) info->pixels += j->npix;
    return SPPM_OK;
}

int sppm_batch_set_stage_timing_mask(sppm_batch* b, uint32_t mask) {
    if (!b) return fail(SPPM_ERR_ARG, "null batch");
    b->rt.timing_mask = mask & ((1u << SPPM_STAGE_COUNT) - 1u);
    return SPPM_OK;
}

int sppm_batch_read_stage_times(sppm_batch* b, float ms[SPPM_STAGE_COUNT], uint32_t launches[SPPM_STAGE_COUNT]) {
    if (!b || !ms || !launches) return fail(SPPM_ERR_ARG, "null argument");
    return b->rt.read_stage_times(ms, launches);
}

int sppm_batch_enable_traversal_counters(sppm_batch* b, int enable) {
    if (!b) return fail(SPPM_ERR_ARG, "null batch");
    b->rt.count_traversal = enable != 0;
    return SPPM_OK;
}

}  // extern "C"

// SPPM render server (include/sppm_server.h): continuous batching over the batch C ABI.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "scene_internal.h"
#include "sppm_server.h"
#include "sppm_texture.h"

using sppm::fail;

namespace {

// a request's own copy of the scene arrays (the caller may free theirs once submit returns)
struct SceneCopy {
    std::vector<float> positions, normals, texcoords, light_cdf, node_bounds;
    std::vector<int32_t> material_ids, light_triangles, node_triangle, order_base, order_miss, material_texture;
    std::vector<sppm_material> materials;
    std::vector<uint8_t> textures;
    sppm_scene s{};

    template <class T>
    static void grab(std::vector<T>& v, const T* p, size_t n) {
        if (p && n) v.assign(p, p + n);
    }
    void copy(const sppm_scene& in) {
        const size_t n = in.num_triangles, nn = in.num_nodes;
        grab(positions, in.positions, n * 9);
        grab(normals, in.normals, n * 9);
        grab(texcoords, in.texcoords, n * 6);
        grab(material_ids, in.material_ids, n);
        grab(materials, in.materials, in.num_materials);
        grab(light_triangles, in.light_triangles, in.num_lights);
        grab(light_cdf, in.light_cdf, in.num_lights);
        grab(node_bounds, in.node_bounds, nn * 6);
        grab(node_triangle, in.node_triangle, nn);
        grab(order_base, in.order_base, nn * 6);
        grab(order_miss, in.order_miss, nn * 6);
        if (in.num_textures) {
            grab(material_texture, in.material_texture, in.num_materials);
            grab(textures, in.textures, (size_t)in.num_textures * SPPM_TEXTURE_RES * SPPM_TEXTURE_RES * 4);
        }
        s = in;
        auto ptr = [](auto& v) { return v.empty() ? nullptr : v.data(); };
        s.positions = ptr(positions);
        s.normals = ptr(normals);
        s.texcoords = ptr(texcoords);
        s.material_ids = ptr(material_ids);
        s.materials = ptr(materials);
        s.light_triangles = ptr(light_triangles);
        s.light_cdf = ptr(light_cdf);
        s.node_bounds = ptr(node_bounds);
        s.node_triangle = ptr(node_triangle);
        s.order_base = ptr(order_base);
        s.order_miss = ptr(order_miss);
        s.material_texture = ptr(material_texture);
        s.textures = ptr(textures);
    }
};

struct Request {
    uint64_t ticket = 0;
    sppm_config cfg{};
    sppm_camera cam{};
    SceneCopy scene;                     // until prepared
    sppm_prepared_scene* prep = nullptr;  // the scene's host-side upload work, done by a worker
    sppm_prepared_state* seeds = nullptr;  // and the job's seeded random-state tables
    bool preparing = false;
    uint64_t bytes = 0;
    uint32_t job = 0;
    sppm_request_info info{};
    std::vector<float> image;
    ~Request() {
        sppm_scene_prepared_destroy(prep);
        sppm_state_prepared_destroy(seeds);
    }
};

double now_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct sppm_server {
    sppm_server_config cfg{};
    sppm_batch* batch = nullptr;
    uint64_t budget = 0;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending;
    std::vector<Request*> running;
    std::map<uint64_t, std::unique_ptr<Request>> requests;  // every request not yet fetched
    uint64_t next_ticket = 1;
    bool stop = false;
    sppm_server_stats stats{};
    std::thread thread;
    // preparation workers: the host-side work of each queued request's scene upload (the
    // traversal layout, the 4-wide tree) runs on these threads while the GPU renders, so that
    // admission only allocates and copies
    std::vector<std::thread> workers;
    std::condition_variable cv_prep;

    void loop();
    void prepare_loop();
    void admit(std::unique_lock<std::mutex>& lk);
    void retire();
};

void sppm_server::prepare_loop() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        Request* r = nullptr;
        cv_prep.wait(lk, [&] {
            if (stop) return true;
            for (Request* q : pending)
                if (!q->prep && !q->preparing) {
                    r = q;
                    return true;
                }
            return false;
        });
        if (stop) return;
        r->preparing = true;
        lk.unlock();
        sppm_prepared_scene* p = nullptr;
        sppm_prepared_state* q = nullptr;
        int st = sppm_scene_prepare(&r->scene.s, &p);
        if (!st) st = sppm_state_prepare(&r->cfg, &q);
        if (!st) r->scene = SceneCopy{};  // only this worker touches the copy while preparing
        lk.lock();
        r->preparing = false;
        if (st) {
            sppm_scene_prepared_destroy(p);
            pending.erase(std::find(pending.begin(), pending.end(), r));
            r->info.state = SPPM_REQUEST_FAILED;
            r->info.status = st;
            r->info.t_done = now_since(t0);
            stats.failed++;
            cv_done.notify_all();
            cv_work.notify_all();  // the next request may now be at the front of the queue
        } else {
            r->prep = p;
            r->seeds = q;
            cv_work.notify_all();
        }
    }
}

void sppm_server::admit(std::unique_lock<std::mutex>& lk) {
    while (!pending.empty() && !stop) {
        Request* r = pending.front();
        if (!r->prep) return;  // its scene is still being prepared (requests are admitted in order)
        sppm_batch_info bi;
        sppm_batch_get_info(batch, &bi);
        if (bi.num_jobs >= bi.max_jobs || bi.bytes_used + r->bytes > budget) return;  // wait for room
        pending.pop_front();
        lk.unlock();
        uint32_t job = 0;
        const int st = sppm_batch_add_job_prepared(batch, &r->cfg, r->prep, r->seeds, &r->cam, &job);
        lk.lock();
        if (st == SPPM_ERR_OOM && !running.empty()) {  // the device had less room than the estimate
            pending.push_front(r);
            return;
        }
        if (st) {
            r->info.state = SPPM_REQUEST_FAILED;
            r->info.status = st;
            r->info.t_done = now_since(t0);
            stats.failed++;
            cv_done.notify_all();
            continue;
        }
        sppm_batch_get_info(batch, &bi);
        stats.bytes_used = bi.bytes_used;
        r->job = job;
        r->info.state = SPPM_REQUEST_RUNNING;
        r->info.t_admit = now_since(t0);
        sppm_scene_prepared_destroy(r->prep);  // uploaded: the host copies are no longer needed
        sppm_state_prepared_destroy(r->seeds);
        r->prep = nullptr;
        r->seeds = nullptr;
        running.push_back(r);
        stats.admitted++;
    }
}

void sppm_server::retire() {
    // called without the lock: only this thread touches the batch and the running jobs' images
    for (Request* r : running) {
        if (r->info.passes_done < r->info.target_passes) continue;
        const size_t n = (size_t)r->info.width * r->info.height * 3;
        r->image.resize(n);
        int st = sppm_batch_read_image(batch, r->job, SPPM_IMAGE_RADIANCE, r->image.data(), n);
        sppm_frame_info fi;
        if (!st) st = sppm_batch_get_frame_info(batch, r->job, &fi);
        sppm_batch_remove_job(batch, r->job);
        std::lock_guard<std::mutex> g(mu);
        r->info.t_done = now_since(t0);
        if (st) {
            r->info.state = SPPM_REQUEST_FAILED;
            r->info.status = st;
            stats.failed++;
        } else {
            r->info.state = SPPM_REQUEST_DONE;
            r->info.photons_emitted = fi.photons_emitted;
            stats.completed++;
            stats.photons += fi.photons_emitted;
        }
    }
    sppm_batch_info bi;
    const int ist = sppm_batch_get_info(batch, &bi);
    std::lock_guard<std::mutex> g(mu);
    if (ist == SPPM_OK) stats.bytes_used = bi.bytes_used;
    running.erase(std::remove_if(running.begin(), running.end(),
                                 [](Request* r) { return r->info.state != SPPM_REQUEST_RUNNING; }),
                  running.end());
    cv_done.notify_all();
}

void sppm_server::loop() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        admit(lk);
        if (stop) break;
        if (running.empty()) {
            cv_work.wait(lk, [&] { return stop || (!pending.empty() && pending.front()->prep); });
            continue;
        }
        // passes until the next job reaches its target (at most passes_per_step)
        uint32_t n = std::max<uint32_t>(cfg.passes_per_step, 1);
        for (Request* r : running) n = std::min(n, r->info.target_passes - r->info.passes_done);
        lk.unlock();
        const auto t = std::chrono::steady_clock::now();
        int st = sppm_batch_run_passes(batch, n);
        if (st) {  // a launch failed: fail every resident request
            lk.lock();
            for (Request* r : running) {
                sppm_batch_remove_job(batch, r->job);
                r->info.state = SPPM_REQUEST_FAILED;
                r->info.status = st;
                r->info.t_done = now_since(t0);
                stats.failed++;
            }
            running.clear();
            cv_done.notify_all();
            continue;
        }
        lk.lock();
        for (Request* r : running) r->info.passes_done += n;
        stats.passes += n;
        const bool any_done = std::any_of(running.begin(), running.end(), [](Request* r) {
            return r->info.passes_done >= r->info.target_passes;
        });
        lk.unlock();
        if (any_done) retire();
        else sppm_batch_synchronize(batch);  // keeps the host within one step of the GPU
        lk.lock();
        stats.busy_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
    }
    // stopping: drop what is resident
    for (Request* r : running) sppm_batch_remove_job(batch, r->job);
    running.clear();
}

extern "C" {

void sppm_server_config_defaults(sppm_server_config* c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    sppm_batch_config_defaults(&c->batch);
    c->passes_per_step = 1;
    c->max_queue = 4096;
}

int sppm_server_create(const sppm_server_config* cfg, int device, sppm_server** out) {
    if (!cfg || !out) return fail(SPPM_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->passes_per_step == 0) return fail(SPPM_ERR_ARG, "passes_per_step must be at least 1");
    std::unique_ptr<sppm_server> s(new (std::nothrow) sppm_server());
    if (!s) return fail(SPPM_ERR_OOM, "host allocation failed");
    s->cfg = *cfg;
    int st = sppm_batch_create(&cfg->batch, device, &s->batch);
    if (st) return st;
    if ((st = sppm_batch_set_tuning(s->batch, &cfg->tuning))) {
        sppm_batch_destroy(s->batch);
        return st;
    }
    sppm_batch_info bi;
    sppm_batch_get_info(s->batch, &bi);
    s->budget = bi.memory_budget;
    s->stats.memory_budget = bi.memory_budget;
    s->t0 = std::chrono::steady_clock::now();
    try {
        const unsigned hw = std::thread::hardware_concurrency();
        const unsigned nw = std::max(1u, std::min(4u, hw / 4));
        for (unsigned k = 0; k < nw; k++) s->workers.emplace_back([p = s.get()] { p->prepare_loop(); });
        s->thread = std::thread([p = s.get()] { p->loop(); });
    } catch (...) {
        {
            std::lock_guard<std::mutex> g(s->mu);
            s->stop = true;
        }
        s->cv_prep.notify_all();
        for (auto& w : s->workers)
            if (w.joinable()) w.join();
        sppm_batch_destroy(s->batch);
        return fail(SPPM_ERR_OOM, "could not start the server threads");
    }
    *out = s.release();
    return SPPM_OK;
}

void sppm_server_destroy(sppm_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->cv_prep.notify_all();
    if (s->thread.joinable()) s->thread.join();
    for (auto& w : s->workers)
        if (w.joinable()) w.join();
    sppm_batch_destroy(s->batch);
    delete s;
}

int sppm_server_submit(sppm_server* s, const sppm_config* cfg, const sppm_scene* scene, const sppm_camera* cam,
                       uint32_t target_passes, uint64_t* ticket) {
    if (!s || !cfg || !scene || !cam || !ticket) return fail(SPPM_ERR_ARG, "null argument");
    if (target_passes == 0) return fail(SPPM_ERR_ARG, "target_passes must be at least 1");
    uint64_t bytes = 0;
    int st = sppm_batch_job_bytes(s->batch, cfg, scene, &bytes);
    if (st) return st;
    if (bytes > s->budget)
        return fail(SPPM_ERR_OOM, "request needs %llu bytes, more than the whole %llu-byte budget",
                    (unsigned long long)bytes, (unsigned long long)s->budget);
    std::unique_ptr<Request> r(new (std::nothrow) Request());
    if (!r) return fail(SPPM_ERR_OOM, "host allocation failed");
    try {
        r->scene.copy(*scene);
    } catch (const std::bad_alloc&) {
        return fail(SPPM_ERR_OOM, "host allocation failed (scene copy)");
    }
    r->cfg = *cfg;
    r->cam = *cam;
    r->bytes = bytes;
    r->info.state = SPPM_REQUEST_QUEUED;
    r->info.target_passes = target_passes;
    r->info.width = cfg->width;
    r->info.height = cfg->height;
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->pending.size() >= s->cfg.max_queue)
            return fail(SPPM_ERR_STATE, "%zu requests are already waiting", s->pending.size());
        r->ticket = s->next_ticket++;
        r->info.t_submit = now_since(s->t0);
        *ticket = r->ticket;
        s->pending.push_back(r.get());
        s->requests[r->ticket] = std::move(r);
        s->stats.submitted++;
    }
    s->cv_prep.notify_one();
    return SPPM_OK;
}

int sppm_server_poll(sppm_server* s, uint64_t ticket, sppm_request_info* info) {
    if (!s || !info) return fail(SPPM_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) return fail(SPPM_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
    *info = it->second->info;
    return SPPM_OK;
}

int sppm_server_wait(sppm_server* s, uint64_t ticket, double timeout_seconds, sppm_request_info* info) {
    if (!s || !info) return fail(SPPM_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) return fail(SPPM_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
    Request* r = it->second.get();
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(std::max(timeout_seconds, 0.0)), [&] {
        return r->info.state == SPPM_REQUEST_DONE || r->info.state == SPPM_REQUEST_FAILED;
    });
    *info = r->info;
    if (!ok) return fail(SPPM_ERR_STATE, "request %llu not finished after %.3f s", (unsigned long long)ticket,
                         timeout_seconds);
    return SPPM_OK;
}

int sppm_server_fetch_image(sppm_server* s, uint64_t ticket, float* rgb, size_t num_floats) {
    if (!s || !rgb) return fail(SPPM_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) return fail(SPPM_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
    Request* r = it->second.get();
    if (r->info.state != SPPM_REQUEST_DONE) return fail(SPPM_ERR_STATE, "request %llu is not done", (unsigned long long)ticket);
    if (num_floats != r->image.size()) return fail(SPPM_ERR_ARG, "image needs %zu floats", r->image.size());
    memcpy(rgb, r->image.data(), num_floats * sizeof(float));
    s->requests.erase(it);
    return SPPM_OK;
}

int sppm_server_get_stats(sppm_server* s, sppm_server_stats* out) {
    if (!s || !out) return fail(SPPM_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    *out = s->stats;
    out->resident = (uint32_t)s->running.size();
    out->queued = (uint32_t)s->pending.size();
    out->memory_budget = s->budget;
    return SPPM_OK;
}

}  // extern "C"

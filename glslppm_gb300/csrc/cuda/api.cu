// C ABI of the SPPM path (include/sppm.h): render contexts, scene packing, pass sequencing.
//
// A context owns one job: its scene in the traversal layout, its camera, its per-pixel and
// per-photon progressive state and its hashed grid, all in one device arena.  A frame is queued
// as the launch sequence of m_display (glslppm.cpp:214-536); the scalars the reference reads back
// between its draws (bounding box, photon count) stay on the device.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "../host/scene_internal.h"
#include "device_common.cuh"
#include "kernels.h"
#include "../host/scene_bvh4.h"

using namespace sppm_dev;
using sppm::fail;

#define SPPM_CK(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(SPPM_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                  \
    } while (0)

namespace {

// bump allocator over one cudaMalloc
struct Arena {
    char* base = nullptr;
    size_t size = 0, used = 0;
    ~Arena() {
        if (base) cudaFree(base);
    }
    static size_t align(size_t n) { return (n + 255) & ~size_t(255); }
    int reserve(size_t bytes) {
        if (base) cudaFree(base);
        base = nullptr;
        used = 0;
        size = bytes;
        if (bytes == 0) return SPPM_OK;
        cudaError_t e = cudaMalloc(&base, bytes);
        if (e != cudaSuccess) {
            base = nullptr;
            size = 0;
            return fail(e == cudaErrorMemoryAllocation ? SPPM_ERR_OOM : SPPM_ERR_CUDA,
                        "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        }
        return SPPM_OK;
    }
    template <class T>
    T* take(size_t count) {
        const size_t b = align(sizeof(T) * count);
        if (used + b > size) return nullptr;
        T* p = reinterpret_cast<T*>(base + used);
        used += b;
        return p;
    }
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
    uint32_t kernels = 0;  // kernel nodes (launches per replay)
    bool counting = false;  // captured with the traversal-counting kernels
    cudaGraphNode_t ev_a[SPPM_STAGE_COUNT] = {}, ev_b[SPPM_STAGE_COUNT] = {};
    void drop() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        *this = FrameGraph{};
    }
};

}  // namespace

struct sppm_ctx {
    sppm_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t W = 0, H = 0, PW = 0, PH = 0, P = 0, npix = 0, hash_num = 0;
    Arena state_mem, scene_mem;
    JobDesc job{};  // host copy of the device descriptor
    JobDesc* d_job = nullptr;
    JobState* d_state = nullptr;
    uint32_t* d_tables = nullptr;  // job_ids[1], prefix_pix[2], prefix_ph[2], prefix_hash[2]
    RayQueue queue{};
    uint32_t trace_blocks = 0;
    float* d_image = nullptr;
    bool have_scene = false, have_camera = false;
    uint32_t frames = 0;  // host mirror of frames queued since reset
    uint64_t kernel_launches = 0;  // kernels launched by sppm_run_passes since creation
    float fixed_radius = 0.0f;
    // stage timing
    uint32_t timing_mask = 0;  // bit k: time stage k
    bool count_traversal = false;
    // frame graphs: [0] photon-only frame, [1] frame with an eye pass
    FrameGraph graphs[2];
    bool capturing = false;
    cudaEvent_t placeholder[2 * SPPM_STAGE_COUNT] = {};
    std::vector<StageEvent> pending;
    std::vector<cudaEvent_t> event_pool;
    float stage_ms[SPPM_STAGE_COUNT] = {0};
    uint32_t stage_launches[SPPM_STAGE_COUNT] = {0};

    LaunchSet set(uint32_t which) const {  // 0 pixels, 1 photons, 2 hash slots
        LaunchSet ls;
        ls.jobs = d_job;
        ls.job_ids = d_tables;
        ls.prefix = d_tables + 1 + 2 * which;
        ls.njobs = 1;
        ls.total = which == 0 ? npix : (which == 1 ? P : hash_num);
        return ls;
    }
    cudaEvent_t get_event() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void drop_graphs() {
        graphs[0].drop();
        graphs[1].drop();
    }
    ~sppm_ctx() {
        if (device >= 0) cudaSetDevice(device);
        drop_graphs();
        for (auto e : placeholder)
            if (e) cudaEventDestroy(e);
        for (auto& p : pending) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        for (auto e : event_pool) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// ---- seeding (RandomizeTextures, glslppm.cpp:77-140) -----------------------------------------
float xorshift_frand(uint32_t* s) {
    const uint32_t t = s[0] ^ (s[0] << 11);
    s[0] = s[1];
    s[1] = s[2];
    s[2] = s[3];
    s[3] = (s[3] ^ (s[3] >> 19)) ^ (t ^ (t >> 8));
    return (float)s[3] * (1.0f / 4294967295.0f);
}

uint32_t mix32(uint32_t h) {  // MurmurHash3 fmix32 finaliser
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

void seed_streams(const sppm_config& cfg, uint32_t npix, uint32_t P, std::vector<float>& eye, std::vector<float>& ph,
                  uint32_t xs[4]) {
    xs[0] = 123456789u;
    xs[1] = 362436069u;
    xs[2] = 521288629u;
    xs[3] = 88675123u;
    if (cfg.seed != 0) {
        for (int k = 0; k < 4; k++) xs[k] ^= mix32(cfg.seed * 4u + (uint32_t)k + 0x9E3779B9u);
        if ((xs[0] | xs[1] | xs[2] | xs[3]) == 0) xs[0] = 1;
    }
    eye.resize((size_t)npix * 4);
    ph.resize((size_t)P * 4);
    if (cfg.seed_mode == SPPM_SEED_XORSHIFT) {
        for (size_t i = 0; i < eye.size(); i += 4)
            for (int k = 3; k >= 0; k--) eye[i + k] = (float)((double)xorshift_frand(xs) * 4194304.0);
        for (size_t i = 0; i < ph.size(); i += 4)
            for (int k = 3; k >= 0; k--) ph[i + k] = (float)((double)xorshift_frand(xs) * 4194304.0);
    } else {
        static const uint32_t mlane[4] = {4194287u, 4194277u, 4194191u, 4194167u};
        for (size_t e = 0; e < (size_t)npix + P; e++) {
            for (int k = 0; k < 4; k++) {
                const uint32_t h = mix32(mix32((uint32_t)e * 4u + (uint32_t)k) ^ mix32(cfg.seed + 0x51ED27u * (e >= npix)));
                const float v = (float)(1u + h % (mlane[k] - 1u));
                if (e < npix) eye[e * 4 + k] = v;
                else ph[(e - npix) * 4 + k] = v;
            }
        }
    }
}

int validate_config(const sppm_config* c) {
    if (!c) return fail(SPPM_ERR_ARG, "null config");
    if (c->width == 0 || c->height == 0 || c->photon_width == 0 || c->photon_height == 0)
        return fail(SPPM_ERR_ARG, "image and photon buffer sizes must be positive");
    if ((uint64_t)c->width * c->height > (1u << 28) || (uint64_t)c->photon_width * c->photon_height > (1u << 28))
        return fail(SPPM_ERR_ARG, "image or photon buffer larger than 2^28 elements");
    if (c->hash_slots > (1u << 28)) return fail(SPPM_ERR_ARG, "hash_slots larger than 2^28");
    if (c->max_path_length == 0 || c->max_path_length > 1024) return fail(SPPM_ERR_ARG, "max_path_length must be 1..1024");
    if (c->precision != SPPM_PRECISION_FP32 && c->precision != SPPM_PRECISION_MIXED)
        return fail(SPPM_ERR_ARG, "unknown precision %u", c->precision);
    if (c->seed_mode > SPPM_SEED_HASH) return fail(SPPM_ERR_ARG, "unknown seed mode %u", c->seed_mode);
    if (c->radius_rule > SPPM_RADIUS_DIAGONAL) return fail(SPPM_ERR_ARG, "unknown radius rule %u", c->radius_rule);
    if (!(c->alpha > 0.0f && c->alpha <= 1.0f)) return fail(SPPM_ERR_ARG, "alpha must be in (0, 1]");
    return SPPM_OK;
}

int upload_tables(sppm_ctx* c) {
    const uint32_t t[7] = {0u, 0u, c->npix, 0u, c->P, 0u, c->hash_num};
    SPPM_CK(cudaMemcpyAsync(c->d_tables, t, sizeof(t), cudaMemcpyHostToDevice, c->stream));
    return SPPM_OK;
}

int upload_job(sppm_ctx* c) {
    SPPM_CK(cudaMemcpyAsync(c->d_job, &c->job, sizeof(JobDesc), cudaMemcpyHostToDevice, c->stream));
    SPPM_CK(cudaStreamSynchronize(c->stream));  // c->job is a host stack-lifetime-independent copy
    return SPPM_OK;
}

int reset_state(sppm_ctx* c) {
    std::vector<float> eye, ph;
    JobState st;
    memset(&st, 0, sizeof(st));
    seed_streams(c->cfg, c->npix, c->P, eye, ph, st.xs);
    const DevPixels& px = c->job.px;
    const DevPhotons& pp = c->job.ph;
    cudaStream_t s = c->stream;
    SPPM_CK(cudaMemcpyAsync(px.rng, eye.data(), eye.size() * 4, cudaMemcpyHostToDevice, s));
    SPPM_CK(cudaMemcpyAsync(pp.rng, ph.data(), ph.size() * 4, cudaMemcpyHostToDevice, s));
    const size_t n4 = (size_t)c->npix * sizeof(float4);
    SPPM_CK(cudaMemsetAsync(px.pos, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.refl, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.nrm, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.emi_n, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.flux_r, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.tri, 0xFF, (size_t)c->npix * 4, s));
    SPPM_CK(cudaMemsetAsync(px.t, 0, (size_t)c->npix * 4, s));
    const size_t p4 = (size_t)c->P * sizeof(float4);
    SPPM_CK(cudaMemsetAsync(pp.pos, 0, p4, s));
    SPPM_CK(cudaMemsetAsync(pp.flux, 0, p4, s));
    SPPM_CK(cudaMemsetAsync(pp.dir, 0, p4, s));
    SPPM_CK(cudaMemsetAsync(pp.hit, 0, (size_t)c->P * sizeof(int2), s));
    SPPM_CK(cudaMemsetAsync(c->job.winner, 0xFF, (size_t)c->hash_num * 4, s));
    SPPM_CK(cudaMemsetAsync(c->job.count, 0, (size_t)c->hash_num * 4, s));
    if (c->job.slots) {
        SPPM_CK(cudaMemsetAsync(c->job.slots, 0, (size_t)c->hash_num * sizeof(SlotRec), s));
        SPPM_CK(cudaMemsetAsync(px.stat_n, 0, (size_t)c->npix * 8, s));
        SPPM_CK(cudaMemsetAsync(px.stat_r2, 0, (size_t)c->npix * 8, s));
        SPPM_CK(cudaMemsetAsync(px.stat_tau, 0, (size_t)c->npix * 24, s));
    }
    st.initial_radius = c->fixed_radius;
    SPPM_CK(cudaMemcpyAsync(c->d_state, &st, sizeof(st), cudaMemcpyHostToDevice, s));
    SPPM_CK(cudaStreamSynchronize(s));  // the host vectors go out of scope
    c->frames = 0;
    return SPPM_OK;
}

// ---- scene packing (CGPURT::CreateTextures, gpurt.cpp:47-552, in the traversal layout) --------
struct Packed {
    std::vector<NodeX> nodes;
    std::vector<float4> isect, shade;
    std::vector<DevMaterial> mats;
    std::vector<float> light_cdf;
    std::vector<int32_t> light_tri;
};

int pack_scene(const sppm_scene* s, Packed& out) {
    if (!s) return fail(SPPM_ERR_ARG, "null scene");
    const uint32_t nt = s->num_triangles, nn = s->num_nodes, nm = s->num_materials, nl = s->num_lights;
    if (nt == 0) return fail(SPPM_ERR_ARG, "scene has no triangles");
    if (nt > (uint32_t)kTriMask) return fail(SPPM_ERR_ARG, "scene has more than 2^30 triangles");
    if (nn != 2 * nt - 1) return fail(SPPM_ERR_ARG, "num_nodes %u must be 2*num_triangles-1 = %u", nn, 2 * nt - 1);
    if (!s->positions || !s->normals || !s->material_ids || !s->materials || nm == 0 || !s->node_bounds ||
        !s->node_triangle || !s->order_base || !s->order_miss)
        return fail(SPPM_ERR_ARG, "scene array missing (positions, normals, materials, BVH)");
    if (nl && (!s->light_triangles || !s->light_cdf)) return fail(SPPM_ERR_ARG, "light table missing");
    if (s->light_area != 0.0f && nl == 0) return fail(SPPM_ERR_ARG, "light_area != 0 with an empty light table");
    out.mats.resize(nm);
    for (uint32_t m = 0; m < nm; m++) {
        const sppm_material& sm = s->materials[m];
        if (sm.brdf < -1 || sm.brdf > 6) return fail(SPPM_ERR_UNSUPPORTED, "material %u: brdf %d not supported", m, sm.brdf);
        DevMaterial& d = out.mats[m];
        memset(&d, 0, sizeof(d));
        d.color[0] = sm.color[0];
        d.color[1] = sm.color[1];
        d.color[2] = sm.color[2];
        d.eta = sm.eta;
        d.brdf = sm.brdf;
        d.g = sm.glossiness;
    }
    out.isect.resize((size_t)nt * 3);
    out.shade.resize((size_t)nt * 6);
    for (uint32_t t = 0; t < nt; t++) {
        const int32_t mi = s->material_ids[t];
        if (mi < 0 || (uint32_t)mi >= nm) return fail(SPPM_ERR_ARG, "triangle %u: material %d out of range", t, mi);
        const float* p = s->positions + (size_t)t * 9;
        const sppm::V3 v0 = sppm::v3(p[0], p[1], p[2]), v1 = sppm::v3(p[3], p[4], p[5]), v2 = sppm::v3(p[6], p[7], p[8]);
        const sppm::V3 e0 = v1 - v0, e1 = v2 - v0;
        float mbits;
        memcpy(&mbits, &mi, 4);
        out.isect[t * 3 + 0] = make_float4(v0.x, v0.y, v0.z, e0.x);
        out.isect[t * 3 + 1] = make_float4(e0.y, e0.z, e1.x, e1.y);
        out.isect[t * 3 + 2] = make_float4(e1.z, mbits, 0.0f, 0.0f);
        // geometric normal normalize(cross(V1-V0, V2-V0)) (eyeraytrace.fs:275)
        const sppm::V3 gn = sppm::normalize3(sppm::cross3(e0, e1));
        // shading normals as the shader decodes them: z = sgn(nz) * sqrt(|1 - x*x - y*y|)
        // with sgn(0) = -1 as gpurt.cpp packs it (eyeraytrace.fs:268-270, gpurt.cpp:35-45, 85)
        float N[9];
        const float* n = s->normals + (size_t)t * 9;
        for (int k = 0; k < 3; k++) {
            const float x = n[k * 3], y = n[k * 3 + 1];
            const float sg = n[k * 3 + 2] > 0.0f ? 1.0f : -1.0f;
            N[k * 3] = x;
            N[k * 3 + 1] = y;
            N[k * 3 + 2] = sg * sppm::sqrt_f32(std::fabs(1.0f - x * x - y * y));
        }
        out.shade[t * 6 + 0] = make_float4(gn.x, gn.y, gn.z, mbits);
        out.shade[t * 6 + 1] = make_float4(v0.x, v0.y, v0.z, v1.x);
        out.shade[t * 6 + 2] = make_float4(v1.y, v1.z, v2.x, v2.y);
        out.shade[t * 6 + 3] = make_float4(v2.z, N[0], N[1], N[2]);
        out.shade[t * 6 + 4] = make_float4(N[3], N[4], N[5], N[6]);
        out.shade[t * 6 + 5] = make_float4(N[7], N[8], 0.0f, 0.0f);
    }
    out.nodes.resize((size_t)6 * nn);
    std::vector<uint8_t> seen(nn);
    for (int o = 0; o < 6; o++) {
        std::fill(seen.begin(), seen.end(), 0);
        for (uint32_t i = 0; i < nn; i++) {
            const int32_t c = s->order_base[(size_t)o * nn + i];
            if (c < 0 || (uint32_t)c >= nn || seen[c])
                return fail(SPPM_ERR_ARG, "ordering %d: node %u has an invalid or repeated base id %d", o, i, c);
            seen[c] = 1;
            const int32_t raw = s->order_miss[(size_t)o * nn + i];
            NodeX& d = out.nodes[(size_t)o * nn + i];
            const float* b = s->node_bounds + (size_t)c * 6;
            d.bmin[0] = b[0];
            d.bmin[1] = b[1];
            d.bmin[2] = b[2];
            d.bmax[0] = b[3];
            d.bmax[1] = b[4];
            d.bmax[2] = b[5];
            d.miss = (raw < 0 || (uint32_t)raw >= nn) ? -1 : raw;
            int32_t tri = s->node_triangle[c];
            if (tri >= (int32_t)nt) return fail(SPPM_ERR_ARG, "node %d: triangle %d out of range", c, tri);
            if (tri >= 0 && s->materials[s->material_ids[tri]].brdf == -1) tri |= kEmitterBit;
            d.tri = tri < 0 ? -1 : tri;
        }
    }
    out.light_cdf.assign(s->light_cdf, s->light_cdf + nl);
    out.light_tri.assign(s->light_triangles, s->light_triangles + nl);
    for (uint32_t l = 0; l < nl; l++)
        if (out.light_tri[l] < 0 || (uint32_t)out.light_tri[l] >= nt)
            return fail(SPPM_ERR_ARG, "light %u: triangle %d out of range", l, out.light_tri[l]);
    return SPPM_OK;
}

template <class T>
int put(Arena& a, const std::vector<T>& v, T** dst, cudaStream_t s) {
    *dst = a.take<T>(std::max<size_t>(v.size(), 1));
    if (!*dst) return fail(SPPM_ERR_OOM, "scene arena exhausted");
    if (!v.empty()) SPPM_CK(cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return SPPM_OK;
}

int launch_check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    return SPPM_OK;
}

}  // namespace

// ================================================================================================
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
    c->cfg = *cfg;
    c->device = device;
    SPPM_CK(cudaSetDevice(device));
    SPPM_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->W = cfg->width;
    c->H = cfg->height;
    c->PW = cfg->photon_width;
    c->PH = cfg->photon_height;
    c->P = c->PW * c->PH;
    c->npix = c->W * c->H;
    c->hash_num = cfg->hash_slots ? cfg->hash_slots : c->P;
    const size_t np = c->npix, P = c->P, hn = c->hash_num;
    size_t bytes = 0;
    bytes += Arena::align(sizeof(JobDesc)) + Arena::align(sizeof(JobState)) + Arena::align(64);
    bytes += 6 * Arena::align(np * 16) + 2 * Arena::align(np * 4) + Arena::align(np * 12);
    bytes += 4 * Arena::align(P * 16) + Arena::align(P * 8);
    bytes += 2 * Arena::align(hn * 4);
    bytes += 3 * Arena::align(P * 16) + Arena::align(64) + Arena::align(P * 4);  // ray queue of the wavefront pass
    const bool binned = !(cfg->flags & SPPM_FLAG_UNBINNED_RAYS);
    if (binned) bytes += Arena::align(P * 8) + Arena::align(P * 4) + Arena::align(kRayBins * 4);
    const bool mixed = cfg->precision == SPPM_PRECISION_MIXED;
    if (mixed) bytes += Arena::align(hn * sizeof(SlotRec)) + 2 * Arena::align(np * 8) + Arena::align(np * 24);
    if ((st = c->state_mem.reserve(bytes))) return st;
    Arena& a = c->state_mem;
    c->d_job = a.take<JobDesc>(1);
    c->d_state = a.take<JobState>(1);
    c->d_tables = a.take<uint32_t>(16);
    JobDesc& J = c->job;
    memset(&J, 0, sizeof(J));
    J.px.pos = a.take<float4>(np);
    J.px.refl = a.take<float4>(np);
    J.px.nrm = a.take<float4>(np);
    J.px.rng = a.take<float4>(np);
    J.px.emi_n = a.take<float4>(np);
    J.px.flux_r = a.take<float4>(np);
    J.px.tri = a.take<int32_t>(np);
    J.px.t = a.take<float>(np);
    c->d_image = a.take<float>(np * 3);
    J.ph.pos = a.take<float4>(P);
    J.ph.flux = a.take<float4>(P);
    J.ph.dir = a.take<float4>(P);
    J.ph.rng = a.take<float4>(P);
    J.ph.hit = a.take<int2>(P);
    J.winner = a.take<uint32_t>(hn);
    J.count = a.take<uint32_t>(hn);
    c->queue.org = a.take<float4>(P);
    c->queue.dir = a.take<float4>(P);
    c->queue.hit = a.take<float4>(P);
    c->queue.counters = a.take<uint32_t>(16);
    c->queue.capacity = c->P;
    c->queue.slow = a.take<uint32_t>(P);
    if (binned) {
        c->queue.key = a.take<uint2>(P);
        c->queue.perm = a.take<uint32_t>(P);
        c->queue.bins = a.take<uint32_t>(kRayBins);
    }
    if (mixed) {
        J.slots = a.take<SlotRec>(hn);
        J.px.stat_n = a.take<double>(np);
        J.px.stat_r2 = a.take<double>(np);
        J.px.stat_tau = a.take<double>(np * 3);
        if (!J.px.stat_tau) return fail(SPPM_ERR_OOM, "state arena sizing error (mixed)");
    }
    {
        int sms = 0;
        SPPM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        c->trace_blocks = (uint32_t)sms * (mixed ? trace_photons4_blocks_per_sm() : trace_photons_blocks_per_sm());
    }
    if (!J.count) return fail(SPPM_ERR_OOM, "state arena sizing error");
    J.state = c->d_state;
    J.image = c->d_image;
    J.W = c->W;
    J.H = c->H;
    J.PW = c->PW;
    J.PH = c->PH;
    J.hash_num = c->hash_num;
    J.max_path = cfg->max_path_length;
    J.eye_interval = cfg->eye_pass_interval;
    J.radius_rule = cfg->radius_rule;
    J.flags = cfg->flags;
    J.precision = cfg->precision;
    J.alpha = cfg->alpha;
    J.footprint = cfg->initial_footprint;
    J.focal = cfg->focal_length;
    J.aperture = cfg->aperture;
    if ((st = upload_tables(c.get()))) return st;
    if ((st = reset_state(c.get()))) return st;
    *out = c.release();
    return SPPM_OK;
}

int sppm_upload_scene(sppm_ctx* c, const sppm_scene* scene) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    SPPM_CK(cudaSetDevice(c->device));
    c->drop_graphs();
    Packed pk;
    int st = pack_scene(scene, pk);
    if (st) return st;
    std::vector<sppm::Node4> nodes4;
    if (c->cfg.precision == SPPM_PRECISION_MIXED) {
        uint32_t depth = 0;
        const int b4 = sppm::build_bvh4(*scene, nodes4, &depth);
        if (b4) return fail(SPPM_ERR_ARG, "4-wide BVH construction failed (%d): inconsistent BVH arrays", b4);
        if (depth > sppm::kBvh4MaxDepth)
            return fail(SPPM_ERR_UNSUPPORTED, "4-wide BVH depth %u exceeds the traversal stack (%u levels)", depth,
                        sppm::kBvh4MaxDepth);
        for (auto& n : nodes4)  // photon rays pass through lights: mark leaf triangles of emitters
            for (int k = 0; k < n.count; k++)
                if (n.child[k] < 0 && n.child[k] != sppm::kChildEmpty) {
                    const int32_t tri = ~n.child[k];
                    if (scene->materials[scene->material_ids[tri]].brdf == -1) n.child[k] = ~(tri | kEmitterBit);
                }
    }
    size_t bytes = Arena::align(pk.nodes.size() * sizeof(NodeX)) + Arena::align(pk.isect.size() * 16) +
                   Arena::align(pk.shade.size() * 16) + Arena::align(pk.mats.size() * sizeof(DevMaterial)) +
                   Arena::align(std::max<size_t>(pk.light_cdf.size(), 1) * 4) +
                   Arena::align(std::max<size_t>(pk.light_tri.size(), 1) * 4) +
                   Arena::align(std::max<size_t>(nodes4.size(), 1) * sizeof(sppm::Node4)) + 1024;
    SPPM_CK(cudaStreamSynchronize(c->stream));
    if ((st = c->scene_mem.reserve(bytes))) return st;
    DevScene& S = c->job.scene;
    NodeX* nodes;
    float4 *isect, *shade;
    DevMaterial* mats;
    float* lcdf;
    int32_t* ltri;
    if ((st = put(c->scene_mem, pk.nodes, &nodes, c->stream))) return st;
    if ((st = put(c->scene_mem, pk.isect, &isect, c->stream))) return st;
    if ((st = put(c->scene_mem, pk.shade, &shade, c->stream))) return st;
    if ((st = put(c->scene_mem, pk.mats, &mats, c->stream))) return st;
    if ((st = put(c->scene_mem, pk.light_cdf, &lcdf, c->stream))) return st;
    if ((st = put(c->scene_mem, pk.light_tri, &ltri, c->stream))) return st;
    sppm::Node4* n4 = nullptr;
    if ((st = put(c->scene_mem, nodes4, &n4, c->stream))) return st;
    S.nodes4 = nodes4.empty() ? nullptr : reinterpret_cast<const Node4Dev*>(n4);
    S.flux_unscale = scene->light_area != 0.0f ? scene->light_area * 3.141592f : 1.0f;
    S.flux_unscale_inv = 1.0f / S.flux_unscale;
    S.nodes = nodes;
    S.tri_isect = isect;
    S.tri_shade = shade;
    S.mats = mats;
    S.light_cdf = lcdf;
    S.light_tri = ltri;
    S.num_nodes = scene->num_nodes;
    S.num_tris = scene->num_triangles;
    S.num_lights = scene->num_lights;
    S.num_mats = scene->num_materials;
    S.light_area = scene->light_area;
    S.light_stride = scene->num_lights ? 1.0f / (float)scene->num_lights : 0.0f;
    // SceneBSphere (glslppm.cpp:388-393)
    const float* mn = scene->bbox_min;
    const float* mx = scene->bbox_max;
    const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    S.bsphere[0] = (mx[0] + mn[0]) * 0.5f;
    S.bsphere[1] = (mx[1] + mn[1]) * 0.5f;
    S.bsphere[2] = (mx[2] + mn[2]) * 0.5f;
    S.bsphere[3] = sppm::sqrt_f32(dx * dx + dy * dy + dz * dz) * 0.5f;
    c->fixed_radius = c->cfg.radius_rule == SPPM_RADIUS_DIAGONAL
                          ? c->cfg.radius_fraction * sppm::sqrt_f32(dx * dx + dy * dy + dz * dz)
                          : 0.0f;
    c->job.fixed_radius = c->fixed_radius;
    c->have_scene = true;
    if ((st = upload_job(c))) return st;
    return reset_state(c);
}

int sppm_set_camera(sppm_ctx* c, const sppm_camera* cam) {
    if (!c || !cam) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->device));
    JobDesc& J = c->job;
    for (int k = 0; k < 3; k++) {
        J.cam_pos[k] = cam->origin[k];
        J.cam_u[k] = cam->u[k];
        J.cam_v[k] = cam->v[k];
        J.cam_w[k] = cam->w[k];
    }
    J.cam_cx = (float)cam->width * 0.5f;
    J.cam_cy = (float)cam->height * 0.5f;
    J.cam_dist = cam->distance;
    c->have_camera = true;
    SPPM_CK(cudaStreamSynchronize(c->stream));
    return upload_job(c);
}

int sppm_reset(sppm_ctx* c) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    SPPM_CK(cudaSetDevice(c->device));
    SPPM_CK(cudaStreamSynchronize(c->stream));
    return reset_state(c);
}

// start or end of a timed stage: while a frame graph is being captured, an event record node
// with a placeholder event; otherwise a pooled event recorded on the stream
static void timed(sppm_ctx* c, int stage, bool start) {
    if (!((c->timing_mask >> stage) & 1u)) return;
    if (c->capturing) {
        cudaEventRecordWithFlags(c->placeholder[2 * stage + (start ? 0 : 1)], c->stream, cudaEventRecordExternal);
        return;
    }
    if (start) {
        StageEvent e{stage, c->get_event(), c->get_event()};
        cudaEventRecord(e.a, c->stream);
        c->pending.push_back(e);
    } else {
        cudaEventRecord(c->pending.back().b, c->stream);
    }
}

}  // extern "C"

namespace {

// the launches of one frame (m_display, glslppm.cpp:214-536) on the context's stream
int enqueue_frame(sppm_ctx* c, bool eye) {
    const LaunchSet pix = c->set(0), pho = c->set(1), hsh = c->set(2);
    timed(c, SPPM_STAGE_FRAME_BEGIN, true);
    launch_frame_begin(hsh, c->queue, c->stream);
    timed(c, SPPM_STAGE_FRAME_BEGIN, false);
    if (eye) {
        timed(c, SPPM_STAGE_EYE, true);
        launch_eye_fp32(pix, c->stream);
        timed(c, SPPM_STAGE_EYE, false);
        timed(c, SPPM_STAGE_GRID, true);
        launch_grid(c->d_job, c->d_tables, 1, c->stream);
        timed(c, SPPM_STAGE_GRID, false);
    }
    const bool mixed = c->cfg.precision == SPPM_PRECISION_MIXED;
    if ((c->cfg.flags & SPPM_FLAG_FUSED_PHOTON) && !mixed) {
        timed(c, SPPM_STAGE_PHOTON, true);
        launch_photon_fp32(pho, c->count_traversal, c->stream);
        timed(c, SPPM_STAGE_PHOTON, false);
    } else {
        timed(c, SPPM_STAGE_PHOTON, true);
        launch_photon_gen_fp32(pho, c->queue, c->stream);
        timed(c, SPPM_STAGE_PHOTON, false);
        if (c->queue.key) {
            timed(c, SPPM_STAGE_RAY_BINS, true);
            launch_ray_bins(c->queue, c->stream);
            timed(c, SPPM_STAGE_RAY_BINS, false);
        }
        timed(c, SPPM_STAGE_PHOTON_TRACE, true);
        if (mixed) launch_trace_photons4(pho, c->queue, c->trace_blocks, c->stream);
        else launch_trace_photons_fp32(pho, c->queue, c->count_traversal, c->trace_blocks, c->stream);
        timed(c, SPPM_STAGE_PHOTON_TRACE, false);
        timed(c, SPPM_STAGE_PHOTON_STORE, true);
        launch_photon_store_fp32(pho, c->queue, c->stream);
        if (mixed) launch_slot_fill(pho, c->queue, c->stream);
        timed(c, SPPM_STAGE_PHOTON_STORE, false);
    }
    timed(c, SPPM_STAGE_GATHER, true);
    if (mixed) launch_gather_mixed(pix, c->stream);
    else launch_gather_fp32(pix, c->stream);
    timed(c, SPPM_STAGE_GATHER, false);
    return launch_check("SPPM frame");
}

int build_frame_graph(sppm_ctx* c, bool eye) {
    FrameGraph& g = c->graphs[eye ? 1 : 0];
    g.drop();
    for (auto& e : c->placeholder)
        if (!e) SPPM_CK(cudaEventCreate(&e));
    SPPM_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    const int st = enqueue_frame(c, eye);
    c->capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (st || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return st ? st : fail(SPPM_ERR_CUDA, "frame graph capture failed: %s", cudaGetErrorString(e));
    }
    g.graph = graph;
    g.mask = c->timing_mask;
    g.counting = c->count_traversal;
    size_t n = 0;
    SPPM_CK(cudaGraphGetNodes(graph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    SPPM_CK(cudaGraphGetNodes(graph, nodes.data(), &n));
    for (cudaGraphNode_t node : nodes) {
        cudaGraphNodeType type;
        SPPM_CK(cudaGraphNodeGetType(node, &type));
        if (type == cudaGraphNodeTypeKernel) g.kernels++;
        if (type != cudaGraphNodeTypeEventRecord) continue;
        cudaEvent_t ev = nullptr;
        SPPM_CK(cudaGraphEventRecordNodeGetEvent(node, &ev));
        for (int k = 0; k < SPPM_STAGE_COUNT; k++) {
            if (ev == c->placeholder[2 * k]) g.ev_a[k] = node;
            if (ev == c->placeholder[2 * k + 1]) g.ev_b[k] = node;
        }
    }
    SPPM_CK(cudaGraphInstantiate(&g.exec, graph, 0));
    return SPPM_OK;
}

int replay_frame_graph(sppm_ctx* c, bool eye) {
    FrameGraph& g = c->graphs[eye ? 1 : 0];
    if (!g.exec || g.mask != c->timing_mask || g.counting != c->count_traversal) {
        const int st = build_frame_graph(c, eye);
        if (st) return st;
    }
    for (int k = 0; k < SPPM_STAGE_COUNT; k++) {
        if (!g.ev_a[k] || !g.ev_b[k]) continue;
        StageEvent se{k, c->get_event(), c->get_event()};
        SPPM_CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, g.ev_a[k], se.a));
        SPPM_CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, g.ev_b[k], se.b));
        c->pending.push_back(se);
    }
    SPPM_CK(cudaGraphLaunch(g.exec, c->stream));
    return SPPM_OK;
}

}  // namespace

extern "C" {

int sppm_run_passes(sppm_ctx* c, uint32_t n) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    if (!c->have_scene || !c->have_camera) return fail(SPPM_ERR_STATE, "upload a scene and set a camera before running passes");
    SPPM_CK(cudaSetDevice(c->device));
    const uint32_t interval = c->cfg.eye_pass_interval ? c->cfg.eye_pass_interval : 1u;
    // the traversal-counting kernels run eagerly (they are a measurement pass)
    const bool graphs = !(c->cfg.flags & SPPM_FLAG_EAGER_LAUNCH) && !c->count_traversal;
    for (uint32_t k = 0; k < n; k++) {
        const bool eye = (c->frames % interval) == 0;
        FrameGraph& g = c->graphs[eye ? 1 : 0];
        if (!graphs && !g.exec) {  // captured (not launched) once to count the frame's kernels
            const int st = build_frame_graph(c, eye);
            if (st) return st;
        }
        const int st = graphs ? replay_frame_graph(c, eye) : enqueue_frame(c, eye);
        if (st) return st;
        c->kernel_launches += g.kernels;
        c->frames++;
    }
    return SPPM_OK;
}

int sppm_synchronize(sppm_ctx* c) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    SPPM_CK(cudaSetDevice(c->device));
    SPPM_CK(cudaStreamSynchronize(c->stream));
    uint32_t err = 0;
    SPPM_CK(cudaMemcpy(&err, &c->d_state->err, 4, cudaMemcpyDeviceToHost));
    if (err & kErrWatchdogTraverse)
        return fail(SPPM_ERR_WATCHDOG, "BVH traversal exceeded its step bound (corrupt or cyclic links)");
    if (err & kErrWatchdogLight) return fail(SPPM_ERR_WATCHDOG, "light-table search exceeded its step bound");
    return SPPM_OK;
}

int sppm_read_image(sppm_ctx* c, uint32_t kind, float* rgb, size_t num_floats) {
    if (!c || !rgb) return fail(SPPM_ERR_ARG, "null argument");
    if (kind > SPPM_IMAGE_DISPLAY) return fail(SPPM_ERR_ARG, "unknown image kind %u", kind);
    if (num_floats != (size_t)c->npix * 3) return fail(SPPM_ERR_ARG, "image needs %zu floats", (size_t)c->npix * 3);
    SPPM_CK(cudaSetDevice(c->device));
    timed(c, SPPM_STAGE_RESOLVE, true);
    if (c->cfg.precision == SPPM_PRECISION_MIXED) launch_resolve_mixed(c->set(0), kind, c->stream);
    else launch_resolve_fp32(c->set(0), kind, c->stream);
    timed(c, SPPM_STAGE_RESOLVE, false);
    int st = launch_check("resolve");
    if (st) return st;
    SPPM_CK(cudaMemcpyAsync(rgb, c->d_image, num_floats * 4, cudaMemcpyDeviceToHost, c->stream));
    return sppm_synchronize(c);
}

static void* state_ptr(const sppm_ctx* c, uint32_t kind, size_t* bytes) {
    const JobDesc& J = c->job;
    const size_t np = c->npix, P = c->P, hn = c->hash_num;
    switch (kind) {
        case SPPM_STATE_HIT_POSITION: *bytes = np * 16; return J.px.pos;
        case SPPM_STATE_HIT_REFLECTANCE: *bytes = np * 16; return J.px.refl;
        case SPPM_STATE_HIT_NORMAL: *bytes = np * 16; return J.px.nrm;
        case SPPM_STATE_EYE_RNG: *bytes = np * 16; return J.px.rng;
        case SPPM_STATE_HIT_TRIANGLE: *bytes = np * 4; return J.px.tri;
        case SPPM_STATE_EMISSION_N: *bytes = np * 16; return J.px.emi_n;
        case SPPM_STATE_FLUX_RADIUS: *bytes = np * 16; return J.px.flux_r;
        case SPPM_STATE_PHOTON_POSITION: *bytes = P * 16; return J.ph.pos;
        case SPPM_STATE_PHOTON_FLUX: *bytes = P * 16; return J.ph.flux;
        case SPPM_STATE_PHOTON_DIRECTION: *bytes = P * 16; return J.ph.dir;
        case SPPM_STATE_PHOTON_RNG: *bytes = P * 16; return J.ph.rng;
        case SPPM_STATE_PHOTON_HIT: *bytes = P * 8; return J.ph.hit;
        case SPPM_STATE_SLOT_WINNER: *bytes = hn * 4; return J.winner;
        case SPPM_STATE_SLOT_COUNT: *bytes = hn * 4; return J.count;
        case SPPM_STATE_HIT_T: *bytes = np * 4; return J.px.t;
        case SPPM_STATE_STATS_N: *bytes = J.px.stat_n ? np * 8 : 0; return J.px.stat_n;
        case SPPM_STATE_STATS_R2: *bytes = J.px.stat_r2 ? np * 8 : 0; return J.px.stat_r2;
        case SPPM_STATE_STATS_TAU: *bytes = J.px.stat_tau ? np * 24 : 0; return J.px.stat_tau;
        default: *bytes = 0; return nullptr;
    }
}

size_t sppm_state_bytes(const sppm_ctx* c, uint32_t kind) {
    if (!c) return 0;
    size_t b = 0;
    return state_ptr(c, kind, &b) ? b : 0;
}

int sppm_read_state(sppm_ctx* c, uint32_t kind, void* dst, size_t bytes) {
    if (!c || !dst) return fail(SPPM_ERR_ARG, "null argument");
    size_t need = 0;
    void* src = state_ptr(c, kind, &need);
    if (!src) return fail(SPPM_ERR_ARG, "state kind %u is not kept by this context", kind);
    if (bytes != need) return fail(SPPM_ERR_ARG, "state kind %u has %zu bytes, %zu requested", kind, need, bytes);
    SPPM_CK(cudaSetDevice(c->device));
    SPPM_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    return sppm_synchronize(c);
}

int sppm_get_frame_info(sppm_ctx* c, sppm_frame_info* fi) {
    if (!c || !fi) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->device));
    JobState st;
    SPPM_CK(cudaMemcpyAsync(&st, c->d_state, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
    SPPM_CK(cudaStreamSynchronize(c->stream));
    memset(fi, 0, sizeof(*fi));
    fi->frames = st.frames_started;
    fi->eye_samples = st.eye_samples;
    fi->photons_emitted = st.num_photons;
    fi->num_photons_f32 = st.num_photons_f32;
    fi->initial_radius = st.initial_radius;
    fi->grid_scale = st.grid_scale;
    for (int k = 0; k < 3; k++) {
        fi->bbox_min[k] = st.bbmin[k];
        fi->bbox_max[k] = st.bbmax[k];
    }
    fi->aa_offset[0] = st.aa[0];
    fi->aa_offset[1] = st.aa[1];
    fi->photon_segments = st.photon_segments;
    fi->eye_segments = st.eye_segments;
    fi->counted_segments = st.count_segments;
    fi->counted_nodes = st.count_nodes;
    fi->counted_triangles = st.count_tris;
    fi->coop_segments = st.coop_segments;
    fi->kernel_launches = c->kernel_launches;
    return SPPM_OK;
}

int sppm_enable_traversal_counters(sppm_ctx* c, int enable) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    c->count_traversal = enable != 0;
    return SPPM_OK;
}

int sppm_enable_stage_timing(sppm_ctx* c, int enable) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    c->timing_mask = enable ? (1u << SPPM_STAGE_COUNT) - 1u : 0u;
    return SPPM_OK;
}

int sppm_set_stage_timing_mask(sppm_ctx* c, uint32_t mask) {
    if (!c) return fail(SPPM_ERR_ARG, "null context");
    c->timing_mask = mask & ((1u << SPPM_STAGE_COUNT) - 1u);
    return SPPM_OK;
}

int sppm_read_stage_times(sppm_ctx* c, float ms[SPPM_STAGE_COUNT], uint32_t launches[SPPM_STAGE_COUNT]) {
    if (!c || !ms || !launches) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->device));
    SPPM_CK(cudaStreamSynchronize(c->stream));
    for (auto& p : c->pending) {
        float t = 0.0f;
        SPPM_CK(cudaEventElapsedTime(&t, p.a, p.b));
        c->stage_ms[p.stage] += t;
        c->stage_launches[p.stage] += 1;
        c->event_pool.push_back(p.a);
        c->event_pool.push_back(p.b);
    }
    c->pending.clear();
    for (int k = 0; k < SPPM_STAGE_COUNT; k++) {
        ms[k] = c->stage_ms[k];
        launches[k] = c->stage_launches[k];
        c->stage_ms[k] = 0.0f;
        c->stage_launches[k] = 0;
    }
    return SPPM_OK;
}

int sppm_time_passes(sppm_ctx* c, uint32_t n, float* ms) {
    if (!c || !ms) return fail(SPPM_ERR_ARG, "null argument");
    SPPM_CK(cudaSetDevice(c->device));
    cudaEvent_t a = c->get_event(), b = c->get_event();
    SPPM_CK(cudaEventRecord(a, c->stream));
    int st = sppm_run_passes(c, n);
    if (st) return st;
    SPPM_CK(cudaEventRecord(b, c->stream));
    SPPM_CK(cudaEventSynchronize(b));
    SPPM_CK(cudaEventElapsedTime(ms, a, b));
    c->event_pool.push_back(a);
    c->event_pool.push_back(b);
    return sppm_synchronize(c);
}

void sppm_destroy(sppm_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
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

int sppm_debug_trace(sppm_ctx* c, const float* org, const float* dir, size_t n, int photon, int cull, int mode,
                     int32_t* tri, float* t) {
    if (!c || !org || !dir || !tri || !t) return fail(SPPM_ERR_ARG, "null argument");
    if (!c->have_scene) return fail(SPPM_ERR_STATE, "upload a scene first");
    if (mode != 0 && mode != 1) return fail(SPPM_ERR_ARG, "mode must be 0 (thread per ray) or 1 (warp per ray)");
    if (n == 0) return SPPM_OK;
    if (n > (1u << 26)) return fail(SPPM_ERR_ARG, "n too large");
    SPPM_CK(cudaSetDevice(c->device));
    SPPM_CK(cudaStreamSynchronize(c->stream));
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
        launch_debug_trace(c->job.scene, d_org, d_dir, (uint32_t)n, photon != 0, cull != 0, mode, d_tri, d_t, d_err,
                           c->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
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

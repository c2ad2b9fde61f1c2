// Render jobs in device memory and the runner that queues the passes of a set of jobs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../host/scene_bvh4.h"
#include "kernels.h"
#include "runtime.h"

using sppm::fail;

namespace sppm_rt {


int Arena::reserve(size_t bytes) {
    release();
    size = bytes;
    if (bytes == 0) return SPPM_OK;
    cudaError_t e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        base = nullptr;
        size = 0;
        return fail(e == cudaErrorMemoryAllocation ? SPPM_ERR_OOM : SPPM_ERR_CUDA, "cudaMalloc(%zu bytes) failed: %s",
                    bytes, cudaGetErrorString(e));
    }
    return SPPM_OK;
}

int launch_check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    return SPPM_OK;
}

void state_to_host_layout(uint32_t kind, void* buf, size_t bytes, uint32_t flags, uint32_t photon_slots) {
    if (kind == SPPM_STATE_SLOT_WINNER) {
        // a slot whose photons were all clipped by the scatter's depth test holds P on the
        // device (the gather reads it as the cleared texel, photon 0); the texture holds no winner
        uint32_t* w = static_cast<uint32_t*>(buf);
        for (size_t i = 0; i < bytes / 4; i++)
            if (w[i] == photon_slots) w[i] = kEmptySlot;
        return;
    }
    if (kind < SPPM_STATE_STATS_N || kind > SPPM_STATE_STATS_TAU) return;
    if (flags & SPPM_FLAG_FP64_STATISTICS) return;  // already IEEE doubles
    char* b = static_cast<char*>(buf);
    for (size_t i = 0; i + 8 <= bytes; i += 8) {
        float pair[2];
        memcpy(pair, b + i, 8);
        const double v = (double)pair[0] + (double)pair[1];  // exact: the pair spans < 53 bits
        memcpy(b + i, &v, 8);
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
    if (c->eye_pass_interval > 4096) return fail(SPPM_ERR_ARG, "eye_pass_interval must be at most 4096");
    if ((c->flags & SPPM_FLAG_FP64_STATISTICS) && c->precision != SPPM_PRECISION_MIXED)
        return fail(SPPM_ERR_ARG, "SPPM_FLAG_FP64_STATISTICS applies to SPPM_PRECISION_MIXED only");
    if ((c->flags & SPPM_FLAG_PHOTON_GRID) && c->precision != SPPM_PRECISION_MIXED)
        return fail(SPPM_ERR_ARG, "SPPM_FLAG_PHOTON_GRID applies to SPPM_PRECISION_MIXED only");
    return SPPM_OK;
}

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
        // the reference's TVector4(rand, rand, rand, rand) evaluates its arguments right to left
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

// ---- scene packing (CGPURT::CreateTextures, gpurt.cpp:47-552, in the traversal layout) --------

int check_scene(const sppm_scene* s) {
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
    return SPPM_OK;
}

int pack_scene(const sppm_scene* s, Packed& out) {
    int st = check_scene(s);
    if (st) return st;
    const uint32_t nt = s->num_triangles, nn = s->num_nodes, nm = s->num_materials, nl = s->num_lights;
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
        out.isect[(size_t)t * 3 + 0] = make_float4(v0.x, v0.y, v0.z, e0.x);
        out.isect[(size_t)t * 3 + 1] = make_float4(e0.y, e0.z, e1.x, e1.y);
        out.isect[(size_t)t * 3 + 2] = make_float4(e1.z, mbits, 0.0f, 0.0f);
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
        out.shade[(size_t)t * 6 + 0] = make_float4(gn.x, gn.y, gn.z, mbits);
        out.shade[(size_t)t * 6 + 1] = make_float4(v0.x, v0.y, v0.z, v1.x);
        out.shade[(size_t)t * 6 + 2] = make_float4(v1.y, v1.z, v2.x, v2.y);
        out.shade[(size_t)t * 6 + 3] = make_float4(v2.z, N[0], N[1], N[2]);
        out.shade[(size_t)t * 6 + 4] = make_float4(N[3], N[4], N[5], N[6]);
        out.shade[(size_t)t * 6 + 5] = make_float4(N[7], N[8], 0.0f, 0.0f);
    }
    out.nodes.resize((size_t)6 * nn);
    out.rank.assign((size_t)6 * nt, 0x7FFFFFFF);
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
            if (tri >= 0) out.rank[(size_t)o * nt + tri] = (int32_t)i;
            if (tri >= 0 && s->materials[s->material_ids[tri]].brdf == -1) tri |= kEmitterBit;
            d.tri = tri < 0 ? -1 : tri;
        }
    }
    out.light_cdf.assign(s->light_cdf, s->light_cdf + nl);
    out.light_tri.assign(s->light_triangles, s->light_triangles + nl);
    for (uint32_t l = 0; l < nl; l++)
        if (out.light_tri[l] < 0 || (uint32_t)out.light_tri[l] >= nt)
            return fail(SPPM_ERR_ARG, "light %u: triangle %d out of range", l, out.light_tri[l]);
    // textures: each material's layer (or -1) and, when any texture coordinate can be used,
    // the triangles' coordinates
    out.mat_layer.assign(nm, -1);
    if (s->num_textures) {
        if (!s->textures || !s->material_texture) return fail(SPPM_ERR_ARG, "texture arrays missing");
        for (uint32_t m = 0; m < nm; m++) {
            const int32_t l = s->material_texture[m];
            if (l < -1 || l >= (int32_t)s->num_textures)
                return fail(SPPM_ERR_ARG, "material %u: texture %d out of range", m, l);
            out.mat_layer[m] = l;
        }
    }
    bool any_tex = false;
    if (s->texcoords)
        for (size_t k = 0; k < (size_t)nt * 6 && !any_tex; k++) any_tex = std::fabs(s->texcoords[k]) < 1e10f;
    if (any_tex) {
        out.tri_tex.resize((size_t)nt * 3);
        for (size_t k = 0; k < (size_t)nt * 3; k++)
            out.tri_tex[k] = make_float2(s->texcoords[k * 2], s->texcoords[k * 2 + 1]);
    }
    return SPPM_OK;
}

template <class T>
int put(Arena& a, const std::vector<T>& v, T** dst, cudaStream_t s) {
    *dst = a.take<T>(std::max<size_t>(v.size(), 1));
    if (!*dst) return fail(SPPM_ERR_OOM, "scene arena exhausted");
    if (!v.empty()) SPPM_CK(cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return SPPM_OK;
}

constexpr size_t kSelfWords = 8;

}  // namespace

// ================================================================================================
// Job
// ================================================================================================
uint64_t Job::state_bytes(const sppm_config& cfg) {
    const size_t np = (size_t)cfg.width * cfg.height, P = (size_t)cfg.photon_width * cfg.photon_height;
    const size_t hn = cfg.hash_slots ? cfg.hash_slots : P;
    size_t b = Arena::align(sizeof(JobState)) + Arena::align(kSelfWords * 4);
    b += 6 * Arena::align(np * 16) + 2 * Arena::align(np * 4) + Arena::align(np * 12);
    b += 4 * Arena::align(P * 16) + Arena::align(P * 8);
    b += 2 * Arena::align(hn * 4);
    if (cfg.precision == SPPM_PRECISION_MIXED)
        b += Arena::align(hn * sizeof(SlotRec)) + 2 * Arena::align(np * 8) + Arena::align(np * 24);
    if (cfg.flags & SPPM_FLAG_PHOTON_GRID) b += Arena::align(P * 8);
    if (cfg.precision == SPPM_PRECISION_FP32) b += Arena::align(3 * kCellTable * 4);
    return b;
}

uint64_t Job::scene_bytes(const sppm_scene& s, uint32_t precision) {
    const uint64_t nt = s.num_triangles, nn = s.num_nodes;
    uint64_t b = Arena::align(6 * nn * sizeof(NodeX)) + Arena::align(nt * 48) + Arena::align(nt * 96) +
                 Arena::align(std::max<uint64_t>(s.num_materials, 1) * sizeof(DevMaterial)) +
                 2 * Arena::align(std::max<uint64_t>(s.num_lights, 1) * 4) + 1024 +
                 Arena::align((uint64_t)s.num_textures * SPPM_TEXTURE_RES * SPPM_TEXTURE_RES * 4) +
                 Arena::align(std::max<uint64_t>(s.num_materials, 1) * 4) + (s.texcoords ? Arena::align(nt * 24) : 0);
    // the 4-wide tree (both precisions: the plain path may trace through it, sppm_tuning.wide_bvh)
    // has at most one node per internal binary node; the triangles' leaf ranks take 24 bytes each
    (void)precision;
    b += Arena::align(std::max<uint64_t>(nn, 1) * sizeof(sppm::Node4)) + Arena::align(6 * nt * 4);
    return b;
}

int Job::init(const sppm_config& c, JobDesc* dd, uint32_t sl, cudaStream_t s) {
    int st = validate_config(&c);
    if (st) return st;
    cfg = c;
    d_desc = dd;
    slot = sl;
    W = c.width;
    H = c.height;
    PW = c.photon_width;
    PH = c.photon_height;
    P = PW * PH;
    npix = W * H;
    hash_num = c.hash_slots ? c.hash_slots : P;
    const size_t np = npix, hn = hash_num;
    if ((st = state_mem.reserve(state_bytes(c)))) return st;
    Arena& a = state_mem;
    d_state = a.take<JobState>(1);
    d_self = a.take<uint32_t>(kSelfWords);
    JobDesc& J = desc;
    memset(&J, 0, sizeof(J));
    J.px.pos = a.take<float4>(np);
    J.px.refl = a.take<float4>(np);
    J.px.nrm = a.take<float4>(np);
    J.px.rng = a.take<float4>(np);
    J.px.emi_n = a.take<float4>(np);
    J.px.flux_r = a.take<float4>(np);
    J.px.tri = a.take<int32_t>(np);
    J.px.t = a.take<float>(np);
    d_image = a.take<float>(np * 3);
    J.ph.pos = a.take<float4>(P);
    J.ph.flux = a.take<float4>(P);
    J.ph.dir = a.take<float4>(P);
    J.ph.rng = a.take<float4>(P);
    J.ph.hit = a.take<int2>(P);
    J.winner = a.take<uint32_t>(hn);
    J.count = a.take<uint32_t>(hn);
    if (c.precision == SPPM_PRECISION_MIXED) {
        J.slots = a.take<SlotRec>(hn);
        J.px.stat_n = a.take<float2>(np);
        J.px.stat_r2 = a.take<float2>(np);
        J.px.stat_tau = a.take<float2>(np * 3);
        if (!J.px.stat_tau) return fail(SPPM_ERR_OOM, "state arena sizing error (mixed)");
    }
    if (c.flags & SPPM_FLAG_PHOTON_GRID) {
        J.grid_key = a.take<uint2>(P);
        if (!J.grid_key) return fail(SPPM_ERR_OOM, "state arena sizing error (photon grid)");
    }
    if (c.precision == SPPM_PRECISION_FP32) {
        J.cell_bounds = a.take<float>(3 * kCellTable);
        if (!J.cell_bounds) return fail(SPPM_ERR_OOM, "state arena sizing error (cell bounds)");
    }
    if (!J.count) return fail(SPPM_ERR_OOM, "state arena sizing error");
    J.state = d_state;
    J.image = d_image;
    J.W = W;
    J.H = H;
    J.PW = PW;
    J.PH = PH;
    J.hash_num = hash_num;
    J.max_path = c.max_path_length;
    J.eye_interval = c.eye_pass_interval;
    J.radius_rule = c.radius_rule;
    J.flags = c.flags;
    J.precision = c.precision;
    J.alpha = c.alpha;
    J.footprint = c.initial_footprint;
    J.focal = c.focal_length;
    J.aperture = c.aperture;
    const uint32_t self[kSelfWords] = {slot, 0u, npix, 0u, P, 0u, hash_num, 0u};
    SPPM_CK(cudaMemcpyAsync(d_self, self, sizeof(self), cudaMemcpyHostToDevice, s));
    if ((st = write_desc(s))) return st;
    return reset(s);
}

Job::~Job() {
    if (copy_ev) {
        if (copy_pending) cudaEventSynchronize(copy_ev);  // the copy reads this job's image
        cudaEventDestroy(copy_ev);
    }
    for (int k = 0; k < 4; k++) {
        if (stage_used[k]) cudaEventSynchronize(stage_ev[k]);
        if (stage_ev[k]) cudaEventDestroy(stage_ev[k]);
    }
    if (stage) cudaFreeHost(stage);
}

// copies the host descriptor into the next of four pinned, mapped staging slots (waiting for the
// slot's previous upload to finish) and returns the slot's device address in *src
int Job::stage_desc(const JobDesc** src) {
    static_assert(sizeof(JobDesc) % 8 == 0, "JobDesc is uploaded in 8-byte words");
    if (!stage) {
        SPPM_CK(cudaHostAlloc(&stage, 4 * sizeof(JobDesc), cudaHostAllocMapped));
        SPPM_CK(cudaHostGetDevicePointer(&stage_dev, stage, 0));
        for (auto& e : stage_ev) SPPM_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const uint32_t k = stage_next & 3u;
    if (stage_used[k]) SPPM_CK(cudaEventSynchronize(stage_ev[k]));
    stage[k] = desc;
    *src = stage_dev + k;
    return SPPM_OK;
}

// marks the slot filled by the last stage_desc as in use until the work queued on s so far is done
int Job::staged(cudaStream_t s) {
    const uint32_t k = stage_next++ & 3u;
    SPPM_CK(cudaEventRecord(stage_ev[k], s));
    stage_used[k] = true;
    return SPPM_OK;
}

// queues the upload of the host descriptor on s through a pinned staging slot (no stream sync)
int Job::write_desc(cudaStream_t s) {
    const JobDesc* src = nullptr;
    int st = stage_desc(&src);
    if (st) return st;
    // read by a kernel straight from the mapped slot: no copy-engine round trip on the stream
    launch_copy_from_host(d_desc, src, sizeof(JobDesc), s);
    SPPM_CK(cudaGetLastError());
    return staged(s);
}

namespace {
// 64-bit fingerprint of byte ranges: four independent multiply-xorshift lanes over 8-byte words
// (a checksum against mix-ups, not a cryptographic hash)
struct Fingerprint {
    uint64_t h[4] = {0x243F6A8885A308D3ull, 0x13198A2E03707344ull, 0xA4093822299F31D0ull, 0x082EFA98EC4E6C89ull};
    static uint64_t mix(uint64_t x) {
        x ^= x >> 31;
        x *= 0x7FB5D329728EA185ull;
        x ^= x >> 27;
        x *= 0x81DADEF4BC2DD44Dull;
        return x ^ (x >> 33);
    }
    void add(const void* p, size_t bytes) {
        const uint8_t* b = static_cast<const uint8_t*>(p);
        size_t i = 0;
        if (b) {
            for (; i + 32 <= bytes; i += 32) {
                uint64_t w[4];
                memcpy(w, b + i, 32);
                for (int k = 0; k < 4; k++) h[k] = (h[k] ^ w[k]) * 0x9E3779B97F4A7C15ull + (h[k] >> 29);
            }
            uint64_t tail[4] = {0, 0, 0, 0};
            memcpy(tail, b + i, bytes - i);
            for (int k = 0; k < 4; k++) h[k] = (h[k] ^ tail[k]) * 0x9E3779B97F4A7C15ull + (h[k] >> 29);
        }
        h[0] ^= mix(bytes + 0x51ED27ull);  // lengths and null pointers count too
    }
    uint64_t value() const { return mix(h[0] ^ mix(h[1] ^ mix(h[2] ^ mix(h[3])))); }
};

uint64_t scene_fingerprint(const sppm_scene& sc) {
    Fingerprint f;
    const size_t n = sc.num_triangles, nn = sc.num_nodes;
    f.add(&sc.num_triangles, 4);
    f.add(sc.positions, n * 36);
    f.add(sc.normals, n * 36);
    f.add(sc.texcoords, sc.texcoords ? n * 24 : 0);
    f.add(sc.material_ids, n * 4);
    f.add(sc.materials, (size_t)sc.num_materials * sizeof(sppm_material));
    f.add(sc.light_triangles, (size_t)sc.num_lights * 4);
    f.add(sc.light_cdf, (size_t)sc.num_lights * 4);
    f.add(&sc.light_area, 4);
    f.add(sc.bbox_min, 12);
    f.add(sc.bbox_max, 12);
    f.add(sc.node_bounds, nn * 24);
    f.add(sc.node_triangle, nn * 4);
    f.add(sc.order_base, nn * 24);
    f.add(sc.order_miss, nn * 24);
    f.add(sc.textures, (size_t)sc.num_textures * SPPM_TEXTURE_RES * SPPM_TEXTURE_RES * 4);
    f.add(sc.material_texture, sc.material_texture ? (size_t)sc.num_materials * 4 : 0);
    return f.value();
}

uint64_t camera_fingerprint(const sppm_camera& c) {
    Fingerprint f;
    f.add(c.origin, 12);
    f.add(c.u, 12);
    f.add(c.v, 12);
    f.add(c.w, 12);
    f.add(&c.distance, 4);
    f.add(&c.width, 4);
    f.add(&c.height, 4);
    return f.value();
}
}  // namespace

int Job::set_camera_desc(const sppm_camera* cam) {
    JobDesc& J = desc;
    for (int k = 0; k < 3; k++) {
        J.cam_pos[k] = cam->origin[k];
        J.cam_u[k] = cam->u[k];
        J.cam_v[k] = cam->v[k];
        J.cam_w[k] = cam->w[k];
    }
    J.cam_cx = (float)cam->width * 0.5f;
    J.cam_cy = (float)cam->height * 0.5f;
    J.cam_dist = cam->distance;
    camera_fp = camera_fingerprint(*cam);
    have_camera = true;
    return SPPM_OK;
}

void prepare_state(const sppm_config& cfg, PreparedState& out) {
    out.npix = cfg.width * cfg.height;
    out.P = cfg.photon_width * cfg.photon_height;
    out.seed = cfg.seed;
    out.seed_mode = cfg.seed_mode;
    seed_streams(cfg, out.npix, out.P, out.eye, out.ph, out.xs);
}

bool PreparedState::matches(const sppm_config& cfg) const {
    return npix == cfg.width * cfg.height && P == cfg.photon_width * cfg.photon_height && seed == cfg.seed &&
           seed_mode == cfg.seed_mode;
}

int Job::reset(cudaStream_t s, const PreparedState* ps) {
    std::vector<float> eye_own, ph_own;
    JobState st;
    memset(&st, 0, sizeof(st));
    if (ps && !ps->matches(cfg)) return fail(SPPM_ERR_ARG, "the prepared state is of another configuration");
    if (ps) memcpy(st.xs, ps->xs, sizeof(st.xs));
    else seed_streams(cfg, npix, P, eye_own, ph_own, st.xs);
    const std::vector<float>& eye = ps ? ps->eye : eye_own;
    const std::vector<float>& ph = ps ? ps->ph : ph_own;
    const DevPixels& px = desc.px;
    const DevPhotons& pp = desc.ph;
    SPPM_CK(cudaMemcpyAsync(px.rng, eye.data(), eye.size() * 4, cudaMemcpyHostToDevice, s));
    SPPM_CK(cudaMemcpyAsync(pp.rng, ph.data(), ph.size() * 4, cudaMemcpyHostToDevice, s));
    const size_t n4 = (size_t)npix * sizeof(float4);
    SPPM_CK(cudaMemsetAsync(px.pos, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.refl, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.nrm, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.emi_n, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.flux_r, 0, n4, s));
    SPPM_CK(cudaMemsetAsync(px.tri, 0xFF, (size_t)npix * 4, s));
    SPPM_CK(cudaMemsetAsync(px.t, 0, (size_t)npix * 4, s));
    const size_t p4 = (size_t)P * sizeof(float4);
    SPPM_CK(cudaMemsetAsync(pp.pos, 0, p4, s));
    SPPM_CK(cudaMemsetAsync(pp.flux, 0, p4, s));
    SPPM_CK(cudaMemsetAsync(pp.dir, 0, p4, s));
    SPPM_CK(cudaMemsetAsync(pp.hit, 0, (size_t)P * sizeof(int2), s));
    SPPM_CK(cudaMemsetAsync(desc.winner, 0xFF, (size_t)hash_num * 4, s));
    SPPM_CK(cudaMemsetAsync(desc.count, 0, (size_t)hash_num * 4, s));
    if (desc.slots) {
        SPPM_CK(cudaMemsetAsync(desc.slots, 0, (size_t)hash_num * sizeof(SlotRec), s));
        SPPM_CK(cudaMemsetAsync(px.stat_n, 0, (size_t)npix * 8, s));
        SPPM_CK(cudaMemsetAsync(px.stat_r2, 0, (size_t)npix * 8, s));
        SPPM_CK(cudaMemsetAsync(px.stat_tau, 0, (size_t)npix * 24, s));
    }
    st.initial_radius = fixed_radius;
    SPPM_CK(cudaMemcpyAsync(d_state, &st, sizeof(st), cudaMemcpyHostToDevice, s));
    SPPM_CK(cudaStreamSynchronize(s));  // the host vectors go out of scope
    return SPPM_OK;
}

int prepare_scene(const sppm_scene* scene, PreparedScene& p) {
    int st = pack_scene(scene, p.pk);
    if (st) return st;
    // both precisions: the plain path may trace through the 4-wide tree too (wide_bvh); a tree the
    // 4-wide walk cannot take is an error for the mixed path only (upload_prepared), the plain path
    // then keeps its binary walk
    p.bvh4_status = sppm::build_bvh4(*scene, p.nodes4, &p.bvh4_depth);
    if (p.bvh4_status || p.bvh4_depth > sppm::kBvh4MaxDepth) p.nodes4.clear();
    for (auto& n : p.nodes4)  // photon rays pass through lights: mark leaf triangles of emitters
        for (int k = 0; k < n.count; k++)
            if (n.child[k] < 0 && n.child[k] != sppm::kChildEmpty) {
                const int32_t tri = ~n.child[k];
                if (scene->materials[scene->material_ids[tri]].brdf == -1) n.child[k] = ~(tri | kEmitterBit);
            }
    if (scene->num_textures)
        p.textures.assign(scene->textures,
                          scene->textures + (size_t)scene->num_textures * SPPM_TEXTURE_RES * SPPM_TEXTURE_RES * 4);
    p.shape = *scene;
    p.shape.positions = p.shape.normals = p.shape.texcoords = p.shape.light_cdf = p.shape.node_bounds = nullptr;
    p.shape.material_ids = p.shape.light_triangles = p.shape.node_triangle = nullptr;
    p.shape.order_base = p.shape.order_miss = p.shape.material_texture = nullptr;
    p.shape.materials = nullptr;
    p.shape.textures = nullptr;
    p.fingerprint = scene_fingerprint(*scene);
    const Packed& pk = p.pk;
    p.device_bytes = Arena::align(pk.nodes.size() * sizeof(NodeX)) + Arena::align(pk.isect.size() * 16) +
                     Arena::align(pk.shade.size() * 16) + Arena::align(pk.mats.size() * sizeof(DevMaterial)) +
                     Arena::align(std::max<size_t>(pk.light_cdf.size(), 1) * 4) +
                     Arena::align(std::max<size_t>(pk.light_tri.size(), 1) * 4) +
                     Arena::align(std::max<size_t>(p.nodes4.size(), 1) * sizeof(sppm::Node4)) + 1024 +
                     Arena::align(pk.tri_tex.size() * sizeof(float2)) + Arena::align(pk.mat_layer.size() * 4) +
                     Arena::align(pk.rank.size() * 4) + Arena::align(p.textures.size());
    return SPPM_OK;
}

int Job::upload_scene(const sppm_scene* scene, cudaStream_t s) {
    PreparedScene p;
    const int st = prepare_scene(scene, p);
    return st ? st : upload_prepared(p, s);
}

int Job::upload_prepared(const PreparedScene& p, cudaStream_t s, const PreparedState* ps) {
    const bool mixed = cfg.precision == SPPM_PRECISION_MIXED;
    if (p.bvh4_status && mixed)
        return fail(SPPM_ERR_ARG, "4-wide BVH construction failed (%d): inconsistent BVH arrays", p.bvh4_status);
    if (p.bvh4_depth > sppm::kBvh4MaxDepth && mixed)
        return fail(SPPM_ERR_UNSUPPORTED, "4-wide BVH depth %u exceeds the traversal stack (%u levels)", p.bvh4_depth,
                    sppm::kBvh4MaxDepth);
    const Packed& pk = p.pk;
    const sppm_scene* scene = &p.shape;
    int st;
    SPPM_CK(cudaStreamSynchronize(s));
    if ((st = scene_mem.reserve(p.device_bytes))) return st;
    scene_bytes_used = p.device_bytes;
    DevScene& S = desc.scene;
    NodeX* nodes;
    float4 *isect, *shade;
    DevMaterial* mats;
    float* lcdf;
    int32_t* ltri;
    if ((st = put(scene_mem, pk.nodes, &nodes, s))) return st;
    if ((st = put(scene_mem, pk.isect, &isect, s))) return st;
    if ((st = put(scene_mem, pk.shade, &shade, s))) return st;
    if ((st = put(scene_mem, pk.mats, &mats, s))) return st;
    if ((st = put(scene_mem, pk.light_cdf, &lcdf, s))) return st;
    if ((st = put(scene_mem, pk.light_tri, &ltri, s))) return st;
    sppm::Node4* n4 = nullptr;
    if ((st = put(scene_mem, p.nodes4, &n4, s))) return st;
    S.nodes4 = p.nodes4.empty() ? nullptr : reinterpret_cast<const Node4Dev*>(n4);
    float2* ttex = nullptr;
    int32_t* mlayer = nullptr;
    if ((st = put(scene_mem, pk.tri_tex, &ttex, s))) return st;
    if ((st = put(scene_mem, pk.mat_layer, &mlayer, s))) return st;
    uint8_t* tex = nullptr;
    if (!p.textures.empty()) {
        tex = scene_mem.take<uint8_t>(p.textures.size());
        if (!tex) return fail(SPPM_ERR_OOM, "scene arena sizing error (textures)");
        SPPM_CK(cudaMemcpyAsync(tex, p.textures.data(), p.textures.size(), cudaMemcpyHostToDevice, s));
    }
    int32_t* rank = nullptr;
    if ((st = put(scene_mem, pk.rank, &rank, s))) return st;
    S.tri_rank = rank;
    S.tri_tex = pk.tri_tex.empty() ? nullptr : ttex;
    S.mat_layer = mlayer;
    S.tex = tex;
    S.mat_rcp = 1.0f / (float)scene->num_materials;
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
    fixed_radius = cfg.radius_rule == SPPM_RADIUS_DIAGONAL
                       ? cfg.radius_fraction * sppm::sqrt_f32(dx * dx + dy * dy + dz * dz)
                       : 0.0f;
    desc.fixed_radius = fixed_radius;
    scene_fp = p.fingerprint;
    have_scene = true;
    if ((st = write_desc(s))) return st;
    return reset(s, ps);
}

int Job::set_camera(const sppm_camera* cam, cudaStream_t s) {
    set_camera_desc(cam);
    return write_desc(s);
}

void* Job::state_ptr(uint32_t kind, size_t* bytes) const {
    const JobDesc& J = desc;
    const size_t np = npix, hn = hash_num, p = P;
    switch (kind) {
        case SPPM_STATE_HIT_POSITION: *bytes = np * 16; return J.px.pos;
        case SPPM_STATE_HIT_REFLECTANCE: *bytes = np * 16; return J.px.refl;
        case SPPM_STATE_HIT_NORMAL: *bytes = np * 16; return J.px.nrm;
        case SPPM_STATE_EYE_RNG: *bytes = np * 16; return J.px.rng;
        case SPPM_STATE_HIT_TRIANGLE: *bytes = np * 4; return J.px.tri;
        case SPPM_STATE_EMISSION_N: *bytes = np * 16; return J.px.emi_n;
        case SPPM_STATE_FLUX_RADIUS: *bytes = np * 16; return J.px.flux_r;
        case SPPM_STATE_PHOTON_POSITION: *bytes = p * 16; return J.ph.pos;
        case SPPM_STATE_PHOTON_FLUX: *bytes = p * 16; return J.ph.flux;
        case SPPM_STATE_PHOTON_DIRECTION: *bytes = p * 16; return J.ph.dir;
        case SPPM_STATE_PHOTON_RNG: *bytes = p * 16; return J.ph.rng;
        case SPPM_STATE_PHOTON_HIT: *bytes = p * 8; return J.ph.hit;
        case SPPM_STATE_SLOT_WINNER: *bytes = hn * 4; return J.winner;
        case SPPM_STATE_SLOT_COUNT: *bytes = hn * 4; return J.count;
        case SPPM_STATE_HIT_T: *bytes = np * 4; return J.px.t;
        case SPPM_STATE_STATS_N: *bytes = J.px.stat_n ? np * 8 : 0; return J.px.stat_n;
        case SPPM_STATE_STATS_R2: *bytes = J.px.stat_r2 ? np * 8 : 0; return J.px.stat_r2;
        case SPPM_STATE_STATS_TAU: *bytes = J.px.stat_tau ? np * 24 : 0; return J.px.stat_tau;
        default: *bytes = 0; return nullptr;
    }
}

int Job::frame_info(sppm_frame_info* fi, cudaStream_t s) const {
    JobState st;
    SPPM_CK(cudaMemcpyAsync(&st, d_state, sizeof(st), cudaMemcpyDeviceToHost, s));
    SPPM_CK(cudaStreamSynchronize(s));
    fill_frame_info(st, fi);
    return SPPM_OK;
}

void fill_frame_info(const JobState& st, sppm_frame_info* fi) {
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
}

namespace {
struct CheckpointHeader {
    char magic[8];
    uint32_t version, W, H, PW, PH, hash_num, precision, state_bytes;
    uint32_t seed_mode, seed;
    uint64_t scene_fp, camera_fp;  // what the job rendered (Job::scene_fp, camera_fp)
};
constexpr char kCheckpointMagic[8] = {'S', 'P', 'P', 'M', 'C', 'K', 'P', '3'};
constexpr uint32_t kCheckpointKinds = SPPM_STATE_STATS_TAU + 1;
}  // namespace

size_t Job::checkpoint_bytes() const {
    size_t b = sizeof(CheckpointHeader) + sizeof(JobState);
    for (uint32_t k = 0; k < kCheckpointKinds; k++) {
        size_t n = 0;
        if (state_ptr(k, &n)) b += n;
    }
    return b;
}

int Job::save_checkpoint(void* dst, size_t bytes, cudaStream_t s) const {
    if (bytes != checkpoint_bytes()) return fail(SPPM_ERR_ARG, "checkpoint needs %zu bytes", checkpoint_bytes());
    char* p = static_cast<char*>(dst);
    CheckpointHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kCheckpointMagic, 8);
    h.version = 2;
    h.W = W;
    h.H = H;
    h.PW = PW;
    h.PH = PH;
    h.hash_num = hash_num;
    h.precision = cfg.precision | (cfg.flags & SPPM_FLAG_FP64_STATISTICS ? 0x100u : 0u);
    h.state_bytes = (uint32_t)sizeof(JobState);
    h.seed_mode = cfg.seed_mode;
    h.seed = cfg.seed;
    h.scene_fp = scene_fp;
    h.camera_fp = camera_fp;
    memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    SPPM_CK(cudaMemcpyAsync(p, d_state, sizeof(JobState), cudaMemcpyDeviceToHost, s));
    p += sizeof(JobState);
    for (uint32_t k = 0; k < kCheckpointKinds; k++) {
        size_t n = 0;
        void* src = state_ptr(k, &n);
        if (!src) continue;
        SPPM_CK(cudaMemcpyAsync(p, src, n, cudaMemcpyDeviceToHost, s));
        p += n;
    }
    SPPM_CK(cudaStreamSynchronize(s));
    return SPPM_OK;
}

int Job::load_checkpoint(const void* src, size_t bytes, cudaStream_t s, uint32_t* frames_started) {
    if (bytes != checkpoint_bytes()) return fail(SPPM_ERR_ARG, "checkpoint has %zu bytes, this job's %zu", bytes,
                                                  checkpoint_bytes());
    const char* p = static_cast<const char*>(src);
    CheckpointHeader h;
    memcpy(&h, p, sizeof(h));
    if (memcmp(h.magic, kCheckpointMagic, 8) != 0 || h.version != 2 || h.state_bytes != sizeof(JobState))
        return fail(SPPM_ERR_ARG, "not a checkpoint of this build");
    const uint32_t prec = cfg.precision | (cfg.flags & SPPM_FLAG_FP64_STATISTICS ? 0x100u : 0u);
    if (h.W != W || h.H != H || h.PW != PW || h.PH != PH || h.hash_num != hash_num || h.precision != prec)
        return fail(SPPM_ERR_ARG, "checkpoint of a %ux%u image with %ux%u photons (%u slots, precision %u) does not "
                    "fit this job", h.W, h.H, h.PW, h.PH, h.hash_num, h.precision);
    if (h.seed_mode != cfg.seed_mode || h.seed != cfg.seed)
        return fail(SPPM_ERR_ARG, "checkpoint of a job seeded with mode %u, seed %u; this job has mode %u, seed %u",
                    h.seed_mode, h.seed, cfg.seed_mode, cfg.seed);
    if (h.scene_fp != scene_fp)
        return fail(SPPM_ERR_ARG, "checkpoint of another scene (scene fingerprint %016llx, this job's %016llx)",
                    (unsigned long long)h.scene_fp, (unsigned long long)scene_fp);
    if (h.camera_fp != camera_fp)
        return fail(SPPM_ERR_ARG, "checkpoint of another camera (camera fingerprint %016llx, this job's %016llx)",
                    (unsigned long long)h.camera_fp, (unsigned long long)camera_fp);
    p += sizeof(h);
    JobState st;
    memcpy(&st, p, sizeof(st));
    p += sizeof(JobState);
    st.cell_table_n = 0;  // the cell-bound table is not in the checkpoint: the next eye pass builds it
    SPPM_CK(cudaStreamSynchronize(s));
    SPPM_CK(cudaMemcpyAsync(d_state, &st, sizeof(st), cudaMemcpyHostToDevice, s));
    for (uint32_t k = 0; k < kCheckpointKinds; k++) {
        size_t n = 0;
        void* dst = state_ptr(k, &n);
        if (!dst) continue;
        SPPM_CK(cudaMemcpyAsync(dst, p, n, cudaMemcpyHostToDevice, s));
        p += n;
    }
    SPPM_CK(cudaStreamSynchronize(s));
    *frames_started = st.frames_started;
    return SPPM_OK;
}

LaunchSet Job::self_set(const JobDesc* table, uint32_t which) const {
    LaunchSet ls{};
    ls.jobs = table;
    ls.job_ids = d_self;
    ls.prefix = d_self + 1 + 2 * which;
    ls.njobs = 1;
    ls.total = which == 0 ? npix : (which == 1 ? P : hash_num);
    return ls;
}

// ================================================================================================
// Runner
// ================================================================================================
void FrameGraph::drop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    *this = FrameGraph{};
}

Runner::~Runner() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    drop_graphs();
    for (auto& p : pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : event_pool) cudaEventDestroy(e);
    for (auto e : placeholder)
        if (e) cudaEventDestroy(e);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (copy) {
        cudaStreamSynchronize(copy);
        cudaStreamDestroy(copy);
    }
    if (resolved_ev) cudaEventDestroy(resolved_ev);
    if (resolve_done) cudaEventDestroy(resolve_done);
    for (auto& t : tickets) cudaEventDestroy(t.ev);
    for (auto e : ticket_pool) cudaEventDestroy(e);
    if (info_host) cudaFreeHost(info_host);
    if (side) {
        cudaStreamSynchronize(side);
        cudaStreamDestroy(side);
    }
    if (stream) cudaStreamDestroy(stream);
}

int Runner::init(int dev, uint32_t prec, uint32_t fl, uint32_t interval, uint32_t jobs_max) {
    device = dev;
    precision = prec;
    flags = fl;
    eye_interval = interval ? interval : 1u;
    max_jobs = jobs_max;
    SPPM_CK(cudaSetDevice(device));
    SPPM_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    SPPM_CK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    SPPM_CK(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    SPPM_CK(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
    SPPM_CK(cudaStreamCreateWithFlags(&copy, cudaStreamNonBlocking));
    SPPM_CK(cudaEventCreateWithFlags(&resolved_ev, cudaEventDisableTiming));
    SPPM_CK(cudaEventCreateWithFlags(&resolve_done, cudaEventDisableTiming));
    SPPM_CK(cudaEventRecord(resolve_done, copy));  // a recorded event from the start
    int st = desc_mem.reserve(Arena::align(sizeof(JobDesc) * std::max<uint32_t>(max_jobs, 1)));
    if (st) return st;
    d_jobs = desc_mem.take<JobDesc>(std::max<uint32_t>(max_jobs, 1));
    int nsm = 0;
    SPPM_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    sms = (uint32_t)nsm;
    trace_fit = precision == SPPM_PRECISION_MIXED ? trace_photons4_blocks_per_sm() : trace_photons_blocks_per_sm();
    trace_fit4 = trace_photons4_blocks_per_sm();
    trace_blocks = sms * trace_fit;
    graphs.resize(eye_interval + 1);
    dirty = true;
    return SPPM_OK;
}

void Runner::drop_graphs() {
    for (auto& g : graphs) g.drop();
}

bool Runner::phase_has_eye(uint32_t phase) const { return phase < eye_pix.size() && eye_pix[phase].njobs > 0; }

int Runner::rebuild() {
    SPPM_CK(cudaSetDevice(device));
    SPPM_CK(cudaStreamSynchronize(stream));
    drop_graphs();
    const uint32_t n = (uint32_t)active.size(), L = eye_interval;
    // launch tables: ids[n], prefix pixels/photons/hash [n+1] each, then per phase the ids and
    // pixel prefix of the jobs that start an eye pass at that phase
    std::vector<uint32_t> t;
    t.reserve(5 * (size_t)n + 4 + (size_t)L * (2 * n + 1));
    uint64_t tot[4] = {0, 0, 0, 0};
    for (Job* j : active) t.push_back(j->slot);
    const size_t pre = t.size();
    // pixels, photon slots, hash slots, and the threads of the pixels in 8x4 tiles (a warp per tile)
    for (int w = 0; w < 4; w++) {
        uint64_t acc = 0;
        for (Job* j : active) {
            t.push_back((uint32_t)acc);
            acc += w == 0 ? j->npix
                 : w == 1 ? j->P
                 : w == 2 ? j->hash_num
                          : 32ull * ((j->W + 7) / 8) * ((j->H + 3) / 4);
        }
        t.push_back((uint32_t)acc);
        tot[w] = acc;
    }
    if (tot[0] > 0xFFFFFFFFull || tot[1] > (1ull << 31) || tot[2] > 0xFFFFFFFFull || tot[3] > 0xFFFFFFFFull)
        return fail(SPPM_ERR_OOM, "jobs exceed 2^32 pixels or hash slots or 2^31 photon slots in one launch");
    std::vector<size_t> eye_off(L), eye_cnt(L);
    for (uint32_t p = 0; p < L; p++) {
        eye_off[p] = t.size();
        std::vector<uint32_t> ids, pref;
        uint64_t acc = 0;
        for (Job* j : active) {
            if (j->eye_phase(L) != p) continue;
            ids.push_back(j->slot);
            pref.push_back((uint32_t)acc);
            acc += j->npix;
        }
        pref.push_back((uint32_t)acc);
        eye_cnt[p] = ids.size();
        t.insert(t.end(), ids.begin(), ids.end());
        t.insert(t.end(), pref.begin(), pref.end());
    }
    int st = table_mem.reserve(Arena::align(std::max<size_t>(t.size(), 1) * 4));
    if (st) return st;
    uint32_t* d_t = table_mem.take<uint32_t>(std::max<size_t>(t.size(), 1));
    SPPM_CK(cudaMemcpy(d_t, t.data(), t.size() * 4, cudaMemcpyHostToDevice));
    auto mk = [&](size_t ids, size_t prefix, uint32_t nj, uint64_t total) {
        LaunchSet ls{};
        ls.jobs = d_jobs;
        ls.job_ids = d_t + ids;
        ls.prefix = d_t + prefix;
        ls.njobs = nj;
        ls.total = (uint32_t)total;
        return ls;
    };
    pix = mk(0, pre, n, tot[0]);
    pho = mk(0, pre + (n + 1), n, tot[1]);
    hsh = mk(0, pre + 2 * (n + 1), n, tot[2]);
    pix_tiles = mk(0, pre + 3 * (n + 1), n, tot[3]);
    eye_pix.assign(L, LaunchSet{});
    eye_ids.assign(L, nullptr);
    for (uint32_t p = 0; p < L; p++) {
        const uint32_t m = (uint32_t)eye_cnt[p];
        uint64_t px = 0;
        for (Job* j : active)
            if (j->eye_phase(L) == p) px += j->npix;
        eye_pix[p] = mk(eye_off[p], eye_off[p] + m, m, px);
        eye_ids[p] = d_t + eye_off[p];
    }
    // the ray queue: one entry per photon slot of every job
    const uint32_t cap = (uint32_t)tot[1];
    if (cap > queue.capacity || !queue.org) {
        const bool binned = !(flags & SPPM_FLAG_UNBINNED_RAYS);
        const size_t c = std::max<uint32_t>(cap, 1);
        size_t bytes = 3 * Arena::align(c * 16) + Arena::align(64) + Arena::align(c * 4) +
                       Arena::align(kEyeDeferred * 4) + Arena::align(c * 4) + Arena::align(c * 16);
        if (binned) bytes += Arena::align(c * 8) + Arena::align(c * 4) + 2 * Arena::align(kRayBins * 4) +
                             Arena::align(kRayBins * 8);
        if ((st = queue_mem.reserve(bytes))) return st;
        Arena& a = queue_mem;
        queue = RayQueue{};
        queue.org = a.take<float4>(c);
        queue.dir = a.take<float4>(c);
        queue.hit = a.take<float4>(c);
        queue.counters = a.take<uint32_t>(16);
        queue.slow = a.take<uint32_t>(c);
        queue.tail_list = a.take<uint32_t>(c);
        queue.tail_state = a.take<float4>(c);
        queue.eye_deferred = a.take<uint32_t>(kEyeDeferred);
        if (binned) {
            queue.key = a.take<uint2>(c);
            queue.perm = a.take<uint32_t>(c);
            queue.bins = a.take<uint32_t>(kRayBins);
            // bins traced in their own order until the first reorder
            queue.bin_rank = a.take<uint32_t>(kRayBins);
            queue.bin_cost = a.take<unsigned long long>(kRayBins);
            std::vector<uint32_t> ident(kRayBins);
            for (uint32_t i = 0; i < kRayBins; i++) ident[i] = i;
            SPPM_CK(cudaMemcpy(queue.bin_rank, ident.data(), kRayBins * 4, cudaMemcpyHostToDevice));
            SPPM_CK(cudaMemset(queue.bin_cost, 0, kRayBins * 8));
        }
        queue.capacity = (uint32_t)c;
        SPPM_CK(cudaMemset(queue.counters, 0, 64));
    }
    // the counting-sort photon grid, when some job uses it: offsets per hash slot (+1), a record
    // per photon slot and the scan's tile sums, for the whole launch
    any_grid = false;
    for (const Job* j : active) any_grid = any_grid || (j->cfg.flags & SPPM_FLAG_PHOTON_GRID) != 0;
    if (any_grid) {
        const uint32_t tiles = grid_tiles((uint32_t)tot[2]);
        const uint64_t need_slots = tot[2] + 1, need_photons = std::max<uint64_t>(tot[1], 1);
        if (need_slots > grid_slots_cap || need_photons > grid_photons_cap || tiles > grid_tiles_cap) {
            const size_t bytes = Arena::align(need_slots * 4) + Arena::align(need_photons * 16) +
                                 Arena::align(std::max<uint32_t>(tiles, 1) * 4);
            grid = PhotonGrid{};
            grid_slots_cap = grid_photons_cap = 0;
            grid_tiles_cap = 0;
            if ((st = grid_mem.reserve(bytes))) return st;
            grid.ofs = grid_mem.take<uint32_t>(need_slots);
            grid.rec = grid_mem.take<uint4>(need_photons);
            grid.tile_sums = grid_mem.take<uint32_t>(std::max<uint32_t>(tiles, 1));
            grid_slots_cap = need_slots;
            grid_photons_cap = need_photons;
            grid_tiles_cap = tiles;
        }
        grid.tiles = tiles;
        grid.rec_capacity = (uint32_t)grid_photons_cap;
    }
    any_slot_records = false;
    for (const Job* j : active)
        any_slot_records = any_slot_records || (j->cfg.precision == SPPM_PRECISION_MIXED &&
                                                !(j->cfg.flags & SPPM_FLAG_PHOTON_GRID));
    dirty = false;
    return SPPM_OK;
}

cudaEvent_t Runner::get_event() {
    if (!event_pool.empty()) {
        cudaEvent_t e = event_pool.back();
        event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// start or end of a timed stage: while a frame graph is being captured, an event record node
// with a placeholder event; otherwise a pooled event recorded on the stream
void Runner::timed(int stage, bool start, cudaStream_t s) {
    if (!((timing_mask >> stage) & 1u)) return;
    if (!s) s = stream;
    if (capturing) {
        cudaEventRecordWithFlags(placeholder[2 * stage + (start ? 0 : 1)], s, cudaEventRecordExternal);
        return;
    }
    if (start) {
        StageEvent e{stage, get_event(), get_event()};
        cudaEventRecord(e.a, s);
        open_stage[stage] = pending.size();
        pending.push_back(e);
    } else {
        cudaEventRecord(pending[open_stage[stage]].b, s);
    }
}

void Runner::wait_resolve(cudaStream_t s) {
    // in a capture, an external event-wait node: each replay waits for the event's last record
    // before the replay's launch
    cudaStreamWaitEvent(s, resolve_done, capturing ? cudaEventWaitExternal : 0);
}

// the launches of one frame (m_display, glslppm.cpp:214-536) for every active job
int Runner::enqueue_frame(uint32_t phase) {
    // the queue as the launches see it: the tuned refill interval, and no bins when the rays are
    // traced in queue order
    RayQueue q = queue;
    q.refill_steps = tune.trace_refill_steps;
    q.tail_lanes = tune.trace_tail_lanes;
    if (tune.unbinned_rays) {
        q.key = nullptr;
        q.perm = nullptr;
        q.bins = nullptr;
        q.bin_rank = nullptr;
        q.bin_cost = nullptr;
    }
    timed(SPPM_STAGE_FRAME_BEGIN, true);
    launch_frame_begin(hsh, q, stream);
    timed(SPPM_STAGE_FRAME_BEGIN, false);
    // the eye pass and the grid it sets run beside the photon generation and traversal (which do
    // not read them); the photon store (hash insertion) waits for the grid
    const bool eye = phase_has_eye(phase);
    const bool mixed = precision == SPPM_PRECISION_MIXED;
    // the plain path through the 4-wide BVH (the same hits): not for the traversal-counting pass,
    // which measures the binary walk
    const bool wide = mixed || (tune.wide_bvh && wide_ok && !count_traversal);
    const uint32_t wide_blocks = std::min(trace_blocks, sms * trace_fit4);
    if (eye) {
        SPPM_CK(cudaEventRecord(fork_ev, stream));
        SPPM_CK(cudaStreamWaitEvent(side, fork_ev, 0));
        wait_resolve(side);  // the eye pass rewrites the emission a pending resolve reads
        timed(SPPM_STAGE_EYE, true, side);
        launch_eye(eye_pix[phase], q, wide, textured, tune.eye_block, side);
        timed(SPPM_STAGE_EYE, false, side);
        timed(SPPM_STAGE_GRID, true, side);
        launch_grid(d_jobs, eye_ids[phase], eye_pix[phase].njobs, side);
        if (!mixed) launch_cell_bounds(d_jobs, eye_ids[phase], eye_pix[phase].njobs, side);
        timed(SPPM_STAGE_GRID, false, side);
        SPPM_CK(cudaEventRecord(join_ev, side));
    }
    if ((flags & SPPM_FLAG_FUSED_PHOTON) && !mixed) {
        if (eye) SPPM_CK(cudaStreamWaitEvent(stream, join_ev, 0));
        timed(SPPM_STAGE_PHOTON, true);
        launch_photon_fp32(pho, count_traversal, textured, stream);
        timed(SPPM_STAGE_PHOTON, false);
    } else {
        // the photon pass in waves of at most tune.photon_wave slots (one wave by default): each
        // wave generates, bins, traces and stores its photons through the ray queue; the hash
        // insertion is a commutative count and an atomic minimum, so the grid is the same for
        // any wave size
        const uint32_t wave = tune.photon_wave && tune.photon_wave < pho.total ? tune.photon_wave : pho.total;
        bool joined = false;
        for (uint32_t first = 0; first < pho.total; first += wave) {
            LaunchSet w = pho;
            w.first = first;
            w.total = pho.total - first > wave ? first + wave : pho.total;
            RayQueue qw = q;
            qw.capacity = w.total - first < q.capacity ? w.total - first : q.capacity;
            if (first) launch_queue_reset(qw, stream);  // k_frame_begin emptied it for the first wave
            // once per eye-pass cycle the bins are reordered by the mean walk of their rays
            else if (eye && qw.key) launch_ray_bins_order(qw, stream);
            timed(SPPM_STAGE_PHOTON, true);
            launch_photon_gen_fp32(w, qw, textured, stream);
            timed(SPPM_STAGE_PHOTON, false);
            if (qw.key) {
                timed(SPPM_STAGE_RAY_BINS, true);
                launch_ray_bins(qw, stream);
                timed(SPPM_STAGE_RAY_BINS, false);
            }
            timed(SPPM_STAGE_PHOTON_TRACE, true);
            if (wide) launch_trace_photons4(pho, qw, mixed ? trace_blocks : wide_blocks, stream);
            else launch_trace_photons_fp32(pho, qw, count_traversal, trace_blocks, stream);
            timed(SPPM_STAGE_PHOTON_TRACE, false);
            if (eye && !joined) {
                SPPM_CK(cudaStreamWaitEvent(stream, join_ev, 0));  // the store needs the eye pass's grid
                joined = true;
            }
            timed(SPPM_STAGE_PHOTON_STORE, true);
            launch_photon_store_fp32(pho, qw, tune.store_block, grid_shift(), stream);
            // the mixed path's slot records are filled after the last wave, inside its store timing
            if (mixed && any_slot_records && w.total == pho.total) launch_slot_fill(hsh, stream);
            timed(SPPM_STAGE_PHOTON_STORE, false);
        }
    }
    if (any_grid) {
        // the counting-sort grid of the pass: every wave's photons are counted and ranked
        grid.shift = grid_shift();
        timed(SPPM_STAGE_PHOTON_SORT, true);
        launch_grid_sort(hsh, pho, grid, stream);
        timed(SPPM_STAGE_PHOTON_SORT, false);
    }
    wait_resolve(stream);  // the gather rewrites the statistics a pending resolve reads
    timed(SPPM_STAGE_GATHER, true);
    if (mixed)
        launch_gather_mixed(any_grid ? pix_tiles : pix, tune.gather_block, fp64_stats, hsh.prefix,
                            any_grid ? &grid : nullptr, stream);
    else launch_gather_fp32(pix, tune.gather_block, stream);
    timed(SPPM_STAGE_GATHER, false);
    return launch_check("SPPM frame");
}

int Runner::build_graph(uint32_t phase, FrameGraph& g) {
    g.drop();
    for (auto& e : placeholder)
        if (!e) SPPM_CK(cudaEventCreate(&e));
    SPPM_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    capturing = true;
    const int st = enqueue_frame(phase);
    capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(stream, &graph);
    if (st || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return st ? st : fail(SPPM_ERR_CUDA, "frame graph capture failed: %s", cudaGetErrorString(e));
    }
    g.graph = graph;
    g.mask = timing_mask;
    g.counting = count_traversal;
    g.textured = textured;
    g.fp64 = fp64_stats;
    g.wide = tune.wide_bvh && wide_ok;
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
            if (ev == placeholder[2 * k]) g.ev_a[k] = node;
            if (ev == placeholder[2 * k + 1]) g.ev_b[k] = node;
        }
    }
    SPPM_CK(cudaGraphInstantiate(&g.exec, graph, 0));
    return SPPM_OK;
}

int Runner::run(uint32_t n) {
    SPPM_CK(cudaSetDevice(device));
    int st;
    if (dirty && (st = rebuild())) return st;
    if (active.empty()) return SPPM_OK;
    // the kernel variants with texture lookups when some job's scene has texture coordinates
    textured = false;
    for (const Job* j : active) textured = textured || j->desc.scene.tri_tex != nullptr;
    fp64_stats = false;
    for (const Job* j : active) fp64_stats = fp64_stats || (j->cfg.flags & SPPM_FLAG_FP64_STATISTICS) != 0;
    wide_ok = true;
    for (const Job* j : active) wide_ok = wide_ok && j->desc.scene.nodes4 != nullptr;
    // the traversal-counting kernels run eagerly (they are a measurement pass)
    const bool use_graphs = !(flags & SPPM_FLAG_EAGER_LAUNCH) && !count_traversal;
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t phase = (uint32_t)(frames % eye_interval);
        FrameGraph& g = graphs[phase_has_eye(phase) ? phase : eye_interval];
        if (!g.exec || g.mask != timing_mask || g.counting != count_traversal || g.textured != textured ||
            g.fp64 != fp64_stats || g.wide != (tune.wide_bvh && wide_ok)) {
            // captured, and launched only in graph mode; eager mode keeps it to count kernels
            if ((st = build_graph(phase, g))) return st;
        }
        if (use_graphs) {
            for (int s = 0; s < SPPM_STAGE_COUNT; s++) {
                if (!g.ev_a[s] || !g.ev_b[s]) continue;
                StageEvent se{s, get_event(), get_event()};
                SPPM_CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, g.ev_a[s], se.a));
                SPPM_CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, g.ev_b[s], se.b));
                pending.push_back(se);
            }
            SPPM_CK(cudaGraphLaunch(g.exec, stream));
        } else if ((st = enqueue_frame(phase))) {
            return st;
        }
        kernel_launches += g.kernels;
        frames++;
    }
    return SPPM_OK;
}

int Runner::synchronize() {
    SPPM_CK(cudaSetDevice(device));
    SPPM_CK(cudaStreamSynchronize(stream));
    SPPM_CK(cudaStreamSynchronize(copy));
    for (auto& t : tickets) ticket_pool.push_back(t.ev);
    tickets.clear();
    std::vector<uint32_t> errs(active.size(), 0);
    for (size_t i = 0; i < active.size(); i++)
        SPPM_CK(cudaMemcpyAsync(&errs[i], &active[i]->d_state->err, 4, cudaMemcpyDeviceToHost, stream));
    SPPM_CK(cudaStreamSynchronize(stream));
    for (size_t i = 0; i < active.size(); i++) {
        if (errs[i] & kErrWatchdogTraverse)
            return fail(SPPM_ERR_WATCHDOG, "job %u: BVH traversal exceeded its step bound (corrupt or cyclic links)",
                        active[i]->slot);
        if (errs[i] & kErrWatchdogLight)
            return fail(SPPM_ERR_WATCHDOG, "job %u: light-table search exceeded its step bound", active[i]->slot);
    }
    return SPPM_OK;
}

int Runner::time(uint32_t n, float* ms) {
    SPPM_CK(cudaSetDevice(device));
    cudaEvent_t a = get_event(), b = get_event();
    SPPM_CK(cudaEventRecord(a, stream));
    int st = run(n);
    if (st) return st;
    SPPM_CK(cudaEventRecord(b, stream));
    SPPM_CK(cudaEventSynchronize(b));
    SPPM_CK(cudaEventElapsedTime(ms, a, b));
    event_pool.push_back(a);
    event_pool.push_back(b);
    return synchronize();
}

static bool block_ok(uint32_t b, uint32_t bound) { return b == 0 || (b >= 32 && b <= bound && b % 32 == 0); }

int Runner::set_tuning(const sppm_tuning* t) {
    if (!t) return fail(SPPM_ERR_ARG, "null tuning");
    if (t->trace_blocks_per_sm > trace_fit)
        return fail(SPPM_ERR_ARG, "trace_blocks_per_sm %u: at most %u traversal blocks fit on an SM",
                    t->trace_blocks_per_sm, trace_fit);
    if (t->trace_refill_steps > 4096) return fail(SPPM_ERR_ARG, "trace_refill_steps %u > 4096", t->trace_refill_steps);
    if (!block_ok(t->eye_block, 128) || !block_ok(t->store_block, 128) || !block_ok(t->gather_block, 256))
        return fail(SPPM_ERR_ARG, "block sizes are 0 or multiples of 32 up to 128 (eye, store) and 256 (gather)");
    if (t->unbinned_rays > 1) return fail(SPPM_ERR_ARG, "unbinned_rays is 0 or 1");
    if (t->photon_wave && t->photon_wave < 1024) return fail(SPPM_ERR_ARG, "photon_wave is 0 or at least 1024");
    if (t->trace_tail_lanes > 32) return fail(SPPM_ERR_ARG, "trace_tail_lanes is 0 (off) .. 32");
    if (t->wide_bvh > 1) return fail(SPPM_ERR_ARG, "wide_bvh is 0 or 1");
    if (t->grid_cell_split > 8 || (t->grid_cell_split & (t->grid_cell_split - 1)))
        return fail(SPPM_ERR_ARG, "grid_cell_split is 0 (default), 1, 2, 4 or 8");
    SPPM_CK(cudaSetDevice(device));
    SPPM_CK(cudaStreamSynchronize(stream));
    tune = *t;
    trace_blocks = sms * (tune.trace_blocks_per_sm ? tune.trace_blocks_per_sm : trace_fit);
    drop_graphs();
    return SPPM_OK;
}

void Runner::get_tuning(sppm_tuning* t) const {
    *t = tune;
    if (!t->trace_blocks_per_sm) t->trace_blocks_per_sm = trace_fit;
    if (!t->trace_refill_steps) t->trace_refill_steps = precision == SPPM_PRECISION_MIXED ? 8u : 32u;
    if (!t->eye_block) t->eye_block = 128;
    if (!t->store_block) t->store_block = 128;
    if (!t->gather_block) t->gather_block = 256;
    if (!t->grid_cell_split) t->grid_cell_split = kDefaultGridCellSplit;
    if (flags & SPPM_FLAG_UNBINNED_RAYS) t->unbinned_rays = 1;  // created without ray bins
}

int Runner::autotune(uint32_t cycles, sppm_tuning* best, float* ms_per_pass) {
    if (!cycles) return fail(SPPM_ERR_ARG, "autotune needs at least one eye-pass cycle per candidate");
    int st;
    SPPM_CK(cudaSetDevice(device));
    if (dirty && (st = rebuild())) return st;
    if (active.empty()) return fail(SPPM_ERR_STATE, "no job to tune on");
    // a window of whole eye-pass cycles holds every phase equally often, wherever it starts
    const uint32_t L = eye_interval, window = cycles * L;
    sppm_tuning cur;
    get_tuning(&cur);
    auto measure = [&](const sppm_tuning& t, float* ms) -> int {
        int e = set_tuning(&t);
        if (e) return e;
        if ((e = run(L))) return e;  // captures the graphs untimed
        return time(window, ms);
    };
    float cur_ms = 0.0f;
    if ((st = measure(cur, &cur_ms))) return st;
    // a grid over ray order x refill interval, then coordinate descent over the other knobs (a
    // second sweep, over all knobs, when the first changed anything); a candidate must beat the
    // best shapes so far by 1 %
    bool changed = false;
    auto knob = [&](uint32_t sppm_tuning::*field, std::vector<uint32_t> values) -> int {
        for (uint32_t v : values) {
            if (v == cur.*field) continue;
            sppm_tuning t = cur;
            t.*field = v;
            float ms = 0.0f;
            const int e = measure(t, &ms);
            if (e) return e;
            if (ms < 0.99f * cur_ms) {
                cur = t;
                cur_ms = ms;
                changed = true;
            }
        }
        return SPPM_OK;
    };
    std::vector<uint32_t> blocks;
    for (uint32_t b : {trace_fit, (3 * trace_fit + 3) / 4, (trace_fit + 1) / 2})
        if (b >= 1 && std::find(blocks.begin(), blocks.end(), b) == blocks.end()) blocks.push_back(b);
    // ray order and refill interval interact: searched together as a grid first.  The plain
    // path's walk stays as set (wide_bvh is the caller's choice, never the tuner's: the 4-wide walk
    // can find a triangle the reference's rounded box test skips, see sppm_tuning.wide_bvh)
    for (uint32_t ub : {0u, 1u}) {
        if (ub && !queue.key) continue;
        for (uint32_t rs : {4u, 8u, 16u, 32u, 64u}) {
            if (ub == cur.unbinned_rays && rs == cur.trace_refill_steps) continue;
            sppm_tuning t = cur;
            t.unbinned_rays = ub;
            t.trace_refill_steps = rs;
            float ms = 0.0f;
            if ((st = measure(t, &ms))) return st;
            if (ms < 0.99f * cur_ms) {
                cur = t;
                cur_ms = ms;
            }
        }
    }
    for (int sweep = 0; sweep < 2; sweep++) {
        changed = false;
        if (sweep && queue.key && (st = knob(&sppm_tuning::unbinned_rays, {0u, 1u}))) return st;
        if (sweep && (st = knob(&sppm_tuning::trace_refill_steps, {4u, 8u, 16u, 32u, 64u}))) return st;
        if ((st = knob(&sppm_tuning::trace_blocks_per_sm, blocks))) return st;
        if ((st = knob(&sppm_tuning::gather_block, {256u, 128u, 64u}))) return st;
        if ((st = knob(&sppm_tuning::store_block, {128u, 64u}))) return st;
        if ((st = knob(&sppm_tuning::eye_block, {128u, 64u}))) return st;
        if (precision == SPPM_PRECISION_FP32 && (st = knob(&sppm_tuning::trace_tail_lanes, {0u, 2u, 8u})))
            return st;
        // wavefront queue depth: the whole pass in one wave, or in 2, 4 or 8 waves
        std::vector<uint32_t> waves = {0u};
        for (uint32_t d : {2u, 4u, 8u})
            if (pho.total / d >= 65536u) waves.push_back((pho.total + d - 1) / d);
        if ((st = knob(&sppm_tuning::photon_wave, waves))) return st;
        if (any_grid && (st = knob(&sppm_tuning::grid_cell_split, {1u, 2u, 4u}))) return st;
        if (!changed) break;
    }
    if ((st = set_tuning(&cur))) return st;
    if (best) *best = cur;
    if (ms_per_pass) *ms_per_pass = cur_ms / (float)window;
    return SPPM_OK;
}

int Runner::read_stage_times(float ms[SPPM_STAGE_COUNT], uint32_t launches[SPPM_STAGE_COUNT]) {
    SPPM_CK(cudaSetDevice(device));
    SPPM_CK(cudaStreamSynchronize(stream));
    for (auto& p : pending) {
        float t = 0.0f;
        SPPM_CK(cudaEventElapsedTime(&t, p.a, p.b));
        stage_ms[p.stage] += t;
        stage_launches[p.stage] += 1;
        event_pool.push_back(p.a);
        event_pool.push_back(p.b);
    }
    pending.clear();
    for (int k = 0; k < SPPM_STAGE_COUNT; k++) {
        ms[k] = stage_ms[k];
        launches[k] = stage_launches[k];
        stage_ms[k] = 0.0f;
        stage_launches[k] = 0;
    }
    return SPPM_OK;
}

int Runner::resolve(Job& j, uint32_t kind, cudaStream_t s) {
    SPPM_CK(cudaSetDevice(device));
    if (!s) s = stream;
    // the image buffer may still be in a copy to host memory (on `copy`, which is in order)
    if (j.copy_pending && s != copy) SPPM_CK(cudaStreamWaitEvent(s, j.copy_ev, 0));
    timed(SPPM_STAGE_RESOLVE, true, s);
    if (precision == SPPM_PRECISION_MIXED) launch_resolve_mixed(j.self_set(d_jobs, 0), kind, s);
    else launch_resolve_fp32(j.self_set(d_jobs, 0), kind, s);
    timed(SPPM_STAGE_RESOLVE, false, s);
    return launch_check("resolve");
}

// at most this many copies in flight: one more waits for the oldest
constexpr size_t kMaxTickets = 16;

int Runner::read_image_async(Job& j, uint32_t kind, float* rgb, size_t bytes, uint64_t* ticket) {
    // the resolve and the copy run on `copy`, after the frames queued so far and beside the next
    // ones, whose eye pass and gather wait for the resolve (resolve_done)
    SPPM_CK(cudaSetDevice(device));
    SPPM_CK(cudaEventRecord(resolved_ev, stream));
    SPPM_CK(cudaStreamWaitEvent(copy, resolved_ev, 0));
    int st = resolve(j, kind, copy);
    if (st) return st;
    SPPM_CK(cudaEventRecord(resolve_done, copy));
    if (!j.copy_ev) SPPM_CK(cudaEventCreateWithFlags(&j.copy_ev, cudaEventDisableTiming));
    if (tickets.size() >= kMaxTickets) {
        SPPM_CK(cudaEventSynchronize(tickets.front().ev));
        ticket_pool.push_back(tickets.front().ev);
        tickets.pop_front();
    }
    cudaEvent_t ev = nullptr;
    if (!ticket_pool.empty()) {
        ev = ticket_pool.back();
        ticket_pool.pop_back();
    } else {
        SPPM_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    SPPM_CK(cudaMemcpyAsync(rgb, j.d_image, bytes, cudaMemcpyDeviceToHost, copy));
    SPPM_CK(cudaEventRecord(j.copy_ev, copy));
    j.copy_pending = true;
    SPPM_CK(cudaEventRecord(ev, copy));
    tickets.push_back(Ticket{next_ticket, ev});
    if (ticket) *ticket = next_ticket;
    next_ticket++;
    return SPPM_OK;
}

int Runner::frame_infos(Job* const* jobs, uint32_t n, sppm_frame_info* out) {
    if (n == 0) return SPPM_OK;
    SPPM_CK(cudaSetDevice(device));
    const uint32_t cap = std::max<uint32_t>(max_jobs, 1);
    if (!info_host) {
        int st = info_mem.reserve(Arena::align(sizeof(JobState) * cap));
        if (st) return st;
        SPPM_CK(cudaMallocHost(&info_host, sizeof(JobState) * cap));
    }
    JobState* d_out = reinterpret_cast<JobState*>(info_mem.base);
    for (uint32_t i0 = 0; i0 < n; i0 += cap) {
        const uint32_t m = std::min(cap, n - i0);
        for (uint32_t c0 = 0; c0 < m; c0 += kStateGatherMax) {
            StateGather list{};
            list.n = std::min<uint32_t>(kStateGatherMax, m - c0);
            for (uint32_t k = 0; k < list.n; k++) list.slot[k] = jobs[i0 + c0 + k]->slot;
            launch_gather_states(d_jobs, list, d_out + c0, stream);
        }
        SPPM_CK(cudaMemcpyAsync(info_host, d_out, sizeof(JobState) * m, cudaMemcpyDeviceToHost, stream));
        SPPM_CK(cudaStreamSynchronize(stream));
        for (uint32_t k = 0; k < m; k++) {
            fill_frame_info(info_host[k], out + i0 + k);
            out[i0 + k].kernel_launches = kernel_launches;
        }
    }
    return launch_check("frame counters");
}

int Runner::image_wait(uint64_t ticket, bool block, int* done) {
    if (ticket == 0 || ticket >= next_ticket) return fail(SPPM_ERR_ARG, "unknown image ticket %llu",
                                                          (unsigned long long)ticket);
    SPPM_CK(cudaSetDevice(device));
    // copies run in ticket order on one stream: once a ticket's event has fired, so have all
    // older ones
    while (!tickets.empty() && tickets.front().id <= ticket) {
        Ticket& t = tickets.front();
        if (block) {
            SPPM_CK(cudaEventSynchronize(t.ev));
        } else {
            const cudaError_t q = cudaEventQuery(t.ev);
            if (q == cudaErrorNotReady) {
                if (done) *done = 0;
                return SPPM_OK;
            }
            if (q != cudaSuccess) return fail(SPPM_ERR_CUDA, "image copy failed: %s", cudaGetErrorString(q));
        }
        ticket_pool.push_back(t.ev);
        tickets.pop_front();
    }
    if (done) *done = 1;
    return SPPM_OK;
}

}  // namespace sppm_rt

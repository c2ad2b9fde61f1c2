/*
 * sppm_oracle.c -- CPU restatement of the glslppm SPPM shader path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The product never links it.
 *
 * It restates, in plain C and in the order the shaders write them, the stages of one SPPM frame
 * of the reference (m_display, glslppm.cpp:214-536):
 *   eyeraytrace.fs   -> oracle_eye_pass       (main :396-554, raytrace :67-290)
 *   max.fs / min.fs  -> bbox of hit positions  (ReduceTexture glslppm.cpp:170-209, :292-311)
 *   photontrace.fs   -> oracle_photon_pass    (main :464-720, raytrace :123-255,
 *                                               GenerateLightSourceSample :345-440, IBL :283-341)
 *   sum.fs           -> emitted-photon count  (glslppm.cpp:396-397)
 *   hash.fs, scatter.vs + depth test, correction.vs + blend -> oracle_hash_build
 *                                              (hash.fs:15-68, scatter.vs:11-23, correction.vs:8-13,
 *                                               glslppm.cpp:404-470)
 *   progressive.fs   -> oracle_gather         (:98-142, AccumulatePhotons :65-95)
 *   re.fs            -> oracle_resolve        (:24-48)
 * Texture addressing is restated as integer indexing: nearest sampling of the texel centres the
 * shaders compute always selects texel k for the k-th element (triangle t's six texels are
 * 6t..6t+5, gpurt.cpp:62-94; node texels are addressed by their canonical index in the block of
 * the ordering, gpurt.cpp:269-470; the light table texel of search step `mid` is mid-1, clamped,
 * photontrace.fs:355-375, restated here with the float texel arithmetic itself).
 *
 * Semantics the GLSL 1.20 specification leaves open are pinned, identically in the CUDA path:
 *   dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z;  cross as in the specification's formula;
 *   normalize(v) = v * (1/sqrt(dot(v,v)));  length = sqrt(dot);  reflect/refract as in the
 *   specification with d = dot(N,I) computed once;  min/max = IEEE minNum/maxNum (fminf/fmaxf);
 *   sign(0) = 0;  fract(x) = x - floor(x);  divisions and square roots correctly rounded;
 *   sin/cos/pow/exp = sppm_fpmath.h;  no fused multiply-add (build with -ffp-contract=off);
 *   cube-map face = major axis, ties broken x before y before z, negative face when the
 *   component is < 0;  the scatter depth test keeps the smallest photon index in a slot and
 *   drops photons with clip-space z >= 1.
 *
 * PARITY PIN: the reference's shaders cannot run here (no OpenGL on either machine).  This
 * restatement is pinned (tests/test_oracle_pin.py) against the reference's own shader sources
 * compiled as C++ through a GLSL-semantics header (oracle/glsl_compat.hpp, built into
 * oracle/_ref/ by oracle/build.py when the reference sources are present), and its host inputs
 * against the reference's host code (oracle/ref_host_dump.cpp).
 *
 * Built twice: single precision (the FP32 checker, bit-exact with the CUDA FP32 path) and, with
 * -DORACLE_FP64, double precision (the converged-image reference for RMSE).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sppm.h"
#include "sppm_fpmath.h"
#include "sppm_texture.h"

#ifdef ORACLE_FP64
typedef double real;
#define RC(x) (x)
#define R_SQRT sqrt
#define R_FLOOR floor
#define R_FABS fabs
#define R_FMIN fmin
#define R_FMAX fmax
#define R_SIN sin
#define R_COS cos
#define R_POW pow
#define R_EXP exp
#define ORACLE_API(name) oracle64_##name
#else
typedef float real;
#define RC(x) (x##f)
#define R_SQRT sqrtf
#define R_FLOOR floorf
#define R_FABS fabsf
#define R_FMIN fminf
#define R_FMAX fmaxf
#define R_SIN sppm_fsin
#define R_COS sppm_fcos
#define R_POW sppm_fpow
#define R_EXP sppm_fexp
#define ORACLE_API(name) oracle32_##name
#endif

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------------------------ */
/* GLSL-like vector helpers with the pinned evaluation order                                   */
/* ------------------------------------------------------------------------------------------ */
typedef struct { real x, y, z; } vec3;
typedef struct { real x, y, z, w; } vec4;

static inline vec3 v3(real x, real y, real z) { vec3 r = {x, y, z}; return r; }
static inline vec3 add3(vec3 a, vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec3 sub3(vec3 a, vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3 mul3(vec3 a, vec3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline vec3 scl3(vec3 a, real s) { return v3(a.x * s, a.y * s, a.z * s); }     /* v * s */
static inline vec3 lscl3(real s, vec3 a) { return v3(s * a.x, s * a.y, s * a.z); }    /* s * v */
static inline vec3 neg3(vec3 a) { return v3(-a.x, -a.y, -a.z); }
static inline real dot3(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline vec3 cross3(vec3 a, vec3 b) {
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline real length3(vec3 a) { return R_SQRT(dot3(a, a)); }
static inline vec3 normalize3(vec3 a) { return scl3(a, RC(1.0) / R_SQRT(dot3(a, a))); }
static inline real len3(vec3 a) { return R_SQRT(dot3(a, a)); }
static inline vec3 reflect3(vec3 i, vec3 n) {
    const real d = RC(2.0) * dot3(n, i);
    return sub3(i, lscl3(d, n));
}
static inline vec3 refract3(vec3 i, vec3 n, real eta) {
    const real d = dot3(n, i);
    const real k = RC(1.0) - eta * eta * (RC(1.0) - d * d);
    if (k < RC(0.0)) return v3(0, 0, 0);
    return sub3(lscl3(eta, i), lscl3(eta * d + R_SQRT(k), n));
}
static inline real signr(real x) { return x > RC(0.0) ? RC(1.0) : (x < RC(0.0) ? RC(-1.0) : RC(0.0)); }
static inline real fractr(real x) { return x - R_FLOOR(x); }
static inline vec3 xyz(vec4 a) { return v3(a.x, a.y, a.z); }
static inline vec4 v4(vec3 a, real w) { vec4 r = {a.x, a.y, a.z, w}; return r; }

/* ------------------------------------------------------------------------------------------ */
/* GPURnd (eyeraytrace.fs:326-347 = photontrace.fs:91-112) and hash (hash.fs:21-48)             */
/* ------------------------------------------------------------------------------------------ */
static const real RND_Q[4] = {RC(1225.0), RC(1585.0), RC(2457.0), RC(2098.0)};
static const real RND_R[4] = {RC(1112.0), RC(367.0), RC(92.0), RC(265.0)};
static const real RND_A[4] = {RC(3423.0), RC(2646.0), RC(1707.0), RC(1999.0)};
static const real RND_M[4] = {RC(4194287.0), RC(4194277.0), RC(4194191.0), RC(4194167.0)};
static real RND_M2[4], RND_MINV[4], RND_QINV[4];

static void rnd_init_constants(void) {
    for (int i = 0; i < 4; i++) {
        RND_M2[i] = RC(0.5) * RND_M[i];       /* vec4(0.5) * m  */
        RND_MINV[i] = RC(1.0) / RND_M[i];     /* vec4(1) / m    */
        RND_QINV[i] = RC(1.0) / RND_Q[i];     /* vec4(1) / q    */
    }
}

/* one Schrage step of the four MLCG lanes; writes the new state, returns (p + beta) * m_ */
static inline void schrage_step(const real in[4], real out[4]) {
    for (int i = 0; i < 4; i++) {
        const real beta = R_FLOOR(in[i] * RND_QINV[i]);
        const real p = RND_A[i] * (in[i] - beta * RND_Q[i]) - beta * RND_R[i];
        const real beta2 = signr(-p) * RND_M2[i] + RND_M2[i];
        out[i] = p + beta2;
    }
}

#ifndef ORACLE_FP64
static inline real gpu_rnd(vec4* n) {
    real s[4] = {n->x, n->y, n->z, n->w}, o[4];
    schrage_step(s, o);
    n->x = o[0];
    n->y = o[1];
    n->z = o[2];
    n->w = o[3];
    const real d = ((o[0] * RND_MINV[0] - o[1] * RND_MINV[1]) + o[2] * RND_MINV[2]) - o[3] * RND_MINV[3];
    return fractr(d);
}

static inline uint32_t hash_cell(vec3 idx, real grid_scale, real hash_scale1, real hash_num) {
    real s[4] = {idx.x * hash_scale1, idx.y * hash_scale1, idx.z * hash_scale1, (grid_scale * RC(0.5)) * hash_scale1};
    real o[4];
    schrage_step(s, o);
    const real d = ((o[0] * RND_MINV[0] - o[1] * RND_MINV[1]) + o[2] * RND_MINV[2]) - o[3] * RND_MINV[3];
    real h = R_FLOOR(fractr(d) * hash_num);
    if (!(h >= RC(0.0))) h = RC(0.0); /* NaN cell (non-finite position) */
    if (h > hash_num - RC(1.0)) h = hash_num - RC(1.0);
    return (uint32_t)h;
}
#else
/* The double-precision oracle draws the single-precision random sequence: GPURnd and the cell
 * hash (both pseudo-random functions of the reference, not part of the estimator's arithmetic) run
 * in single precision exactly as in the FP32 build.  An FP64 render therefore consumes the same
 * random numbers as an FP32 render of the same seed, and the two images differ only through the
 * precision of the light transport and of the estimator (a flipped comparison changes what follows
 * on that path), not through independent samples. */
static float RNDF_Q[4], RNDF_R[4], RNDF_A[4], RNDF_M2[4], RNDF_MINV[4], RNDF_QINV[4];
static int rndf_ready = 0;

static void rndf_init(void) {
    if (rndf_ready) return;
    static const float q[4] = {1225.0f, 1585.0f, 2457.0f, 2098.0f};
    static const float r[4] = {1112.0f, 367.0f, 92.0f, 265.0f};
    static const float a[4] = {3423.0f, 2646.0f, 1707.0f, 1999.0f};
    static const float m[4] = {4194287.0f, 4194277.0f, 4194191.0f, 4194167.0f};
    for (int i = 0; i < 4; i++) {
        RNDF_Q[i] = q[i];
        RNDF_R[i] = r[i];
        RNDF_A[i] = a[i];
        RNDF_M2[i] = 0.5f * m[i];
        RNDF_MINV[i] = 1.0f / m[i];
        RNDF_QINV[i] = 1.0f / q[i];
    }
    rndf_ready = 1;
}

static inline void schrage_step_f32(const float in[4], float out[4]) {
    for (int i = 0; i < 4; i++) {
        const float beta = floorf(in[i] * RNDF_QINV[i]);
        const float p = RNDF_A[i] * (in[i] - beta * RNDF_Q[i]) - beta * RNDF_R[i];
        const float sg = -p > 0.0f ? 1.0f : (-p < 0.0f ? -1.0f : 0.0f);
        out[i] = p + (sg * RNDF_M2[i] + RNDF_M2[i]);
    }
}

static inline float rnd_fold_f32(const float o[4]) {
    return ((o[0] * RNDF_MINV[0] - o[1] * RNDF_MINV[1]) + o[2] * RNDF_MINV[2]) - o[3] * RNDF_MINV[3];
}

static inline real gpu_rnd(vec4* n) {
    rndf_init();
    float s[4] = {(float)n->x, (float)n->y, (float)n->z, (float)n->w}, o[4];
    schrage_step_f32(s, o);
    n->x = o[0];
    n->y = o[1];
    n->z = o[2];
    n->w = o[3];
    const float d = rnd_fold_f32(o);
    return (real)(d - floorf(d));
}

static inline uint32_t hash_cell(vec3 idx, real grid_scale, real hash_scale1, real hash_num) {
    (void)hash_scale1;
    rndf_init();
    const float G = (float)grid_scale;
    const float hs1 = 4194304.0f / G;
    float s[4] = {(float)idx.x * hs1, (float)idx.y * hs1, (float)idx.z * hs1, (G * 0.5f) * hs1};
    float o[4];
    schrage_step_f32(s, o);
    const float d = rnd_fold_f32(o);
    const float hn = (float)hash_num;
    float h = floorf((d - floorf(d)) * hn);
    if (!(h >= 0.0f)) h = 0.0f;
    if (h > hn - 1.0f) h = hn - 1.0f;
    return (uint32_t)h;
}
#endif

/* ------------------------------------------------------------------------------------------ */
/* scene in the reference's packed form                                                        */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    uint32_t nt, nm, nl, nn;
    vec4* tv;     /* [nt][3] (px, py, pz, tx)                                 gpurt.cpp:62-80 */
    vec4* tn;     /* [nt][3] (nx, ny, sgn(nz)*(mat+1), ty)                    gpurt.cpp:82-88 */
    vec4* mat;    /* [nm][2] (r,g,b,eta), (brdf, g, 0, 0)                      gpurt.cpp:109-132 */
    int32_t* light_tri;
    real* light_cdf;
    real light_area;
    real light_stride;                 /* 1 / lightsCDF.size() (glslppm.cpp:381) */
    real bsphere[4];                   /* SceneBSphere (glslppm.cpp:388-393) */
    real* nb;                          /* [nn][6] canonical node min/max */
    int32_t* ntri;                     /* [nn] */
    int32_t* hit_link;                 /* [6][nn] canonical -> canonical or -1 (gpurt.cpp:332-366) */
    int32_t* miss_link;                /* [6][nn] */
    /* material textures (VolumeTextureTextures, gpurt.cpp:158-198; sampling: sppm_texture.h) */
    uint8_t* tex;                      /* [layers][512][512][4] or NULL */
    int32_t* mat_layer;                /* [nm]: layer of the material or -1 (magenta) */
    float mat_rcp;                     /* MaterialNumRcp = 1 / materials (glslppm.cpp:256, 376) */
    int any_tex;                       /* some texture coordinate is below 1e10 (else no lookups) */
} oscene;

typedef struct oracle_ctx {
    sppm_config cfg;
    sppm_camera cam;
    oscene sc;
    uint32_t W, H, PW, PH, P, hash_num;
    /* per pixel (the six MRTs of the eye pass and the two of the progressive pass) */
    vec4 *q_pos, *q_refl, *q_nrm, *q_rng, *q_emi_n, *q_flux_r;
    int32_t* q_tri;
    real* q_t;
    /* per photon slot */
    vec4 *p_pos, *p_flux, *p_dir, *p_rng;
    int32_t *p_tri, *p_depth;
    real* p_t;
    uint8_t* p_emitted;
    /* hash table */
    uint32_t *winner, *count;
    /* counting-sort photon grid (SPPM_FLAG_PHOTON_GRID): photon ids by hash slot, ascending */
    uint32_t *g_ofs, *g_ids, *g_cur;
    /* frame state */
    uint32_t frame, eye_samples;
    uint32_t xs[4];
    real aa[2];
    real bbmin[3], bbmax[3];
    real initial_radius, grid_scale;
    float num_photons_f32;
    uint64_t num_photons;
    uint64_t photon_segments, eye_segments;
    int err;
} oracle_ctx;

static inline vec3 tri_vertex(const oscene* s, int32_t t, int k) { return xyz(s->tv[t * 3 + k]); }
/* N.z = sign(N.z) * sqrt(abs(1 - N.x*N.x - N.y*N.y)) (eyeraytrace.fs:268-270) */
static inline vec3 tri_normal(const oscene* s, int32_t t, int k) {
    const vec4 n = s->tn[t * 3 + k];
    return v3(n.x, n.y, signr(n.z) * R_SQRT(R_FABS(RC(1.0) - n.x * n.x - n.y * n.y)));
}
static inline int32_t tri_material(const oscene* s, int32_t t) {
    return (int32_t)(R_FABS(s->tn[t * 3].z) - RC(1.0));
}

/* ------------------------------------------------------------------------------------------ */
/* traversal                                                                                   */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    real t;
    vec3 pos, nrm, gnrm, col;
    real texu, texv; /* Result.tex (eyeraytrace.fs:280) */
    int brdf;
    real eta, g;
    int32_t matid;
} Isect;

/* col *= texture3D(VolumeTextureTextures, vec3(tex, r)).rgb when |tex.x| < 1e10 (eyeraytrace.fs:443-446,
   photontrace.fs:418-422, 562-565) */
static vec3 tex_modulate(const oscene* s, real tu, real tv, float r, vec3 col) {
    if (!(R_FABS(tu) < RC(1e+10))) return col;
    float t[3];
    sppm_tex_sample(s->tex, s->mat_layer, s->nm, (float)tu, (float)tv, r, t);
    return v3(col.x * (real)t[0], col.y * (real)t[1], col.z * (real)t[2]);
}

typedef struct {
    int32_t tri;
    int32_t mat;
    real t;
} LastIsect;

static inline int cube_face(vec3 d) {
    const real ax = R_FABS(d.x), ay = R_FABS(d.y), az = R_FABS(d.z);
    if (ax >= ay && ax >= az) return d.x < RC(0.0) ? 1 : 0;
    if (ay >= az) return d.y < RC(0.0) ? 3 : 2;
    return d.z < RC(0.0) ? 5 : 4;
}

/* raytrace() of eyeraytrace.fs:67-290 (photon = 0, with cull flag) and photontrace.fs:123-255
   (photon = 1: t bound 1e30, emitters skipped, isect.x >= 0 test) */
static Isect raytrace(oracle_ctx* c, vec3 org, vec3 dir, int photon, int cull, LastIsect* last) {
    const oscene* s = &c->sc;
    Isect r;
    memset(&r, 0, sizeof(r));
    r.t = RC(1.0e+30);
    r.matid = -1;
    r.texu = r.texv = RC(1.0e+30);
    LastIsect is = {-1, -1, photon ? RC(1.0e30) : RC(1.0e20)};
    real bu = 0, bv = 0, bw = 0; /* Barycentric = uvt.ywx -> (v, w, u) */
    const int face = cube_face(dir);
    const vec3 rcp = v3(RC(1.0) / dir.x, RC(1.0) / dir.y, RC(1.0) / dir.z);
    const vec3 t0 = mul3(neg3(rcp), org);
    int32_t node = 0;
    uint32_t steps = 0;
    for (;;) {
        if (++steps > s->nn + 1) {
            c->err = SPPM_ERR_WATCHDOG;
            break;
        }
        const real* b = &s->nb[(size_t)node * 6];
        const vec3 lo = add3(mul3(rcp, v3(b[0], b[1], b[2])), t0);
        const vec3 hi = add3(mul3(rcp, v3(b[3], b[4], b[5])), t0);
        const vec3 a = v3(R_FMIN(lo.x, hi.x), R_FMIN(lo.y, hi.y), R_FMIN(lo.z, hi.z));
        const vec3 bb = v3(R_FMAX(lo.x, hi.x), R_FMAX(lo.y, hi.y), R_FMAX(lo.z, hi.z));
        const real tmin = R_FMAX(R_FMAX(a.x, a.y), a.z);
        const real tmax = R_FMIN(R_FMIN(bb.x, bb.y), bb.z);
        const int hit = (tmin <= tmax) && (tmin <= is.t) && (tmax >= RC(0.0));
        const int32_t tri = s->ntri[node];
        if (tri >= 0 && hit) {
            const vec3 V0 = tri_vertex(s, tri, 0), V1 = tri_vertex(s, tri, 1), V2 = tri_vertex(s, tri, 2);
            const int32_t mi = tri_material(s, tri);
            const int brdf = (int)s->mat[mi * 2 + 1].x;
            const vec3 e0 = sub3(V1, V0), e1 = sub3(V2, V0);
            const vec3 pv = cross3(dir, e1);
            const real det = dot3(e0, pv);
            if (photon || (cull && (det > RC(1e-10))) || !cull) {
                const vec3 tv = sub3(org, V0);
                const vec3 qv = cross3(tv, e0);
                const real u = dot3(tv, pv) / det;
                const real v = dot3(dir, qv) / det;
                const real t = dot3(e1, qv) / det;
                const real w = RC(1.0) - u - v;
                if (u >= RC(0.0) && v >= RC(0.0) && t >= RC(0.0) && w >= RC(0.0) && t < is.t &&
                    (!photon || brdf != -1)) {
                    bu = v;
                    bv = w;
                    bw = u;
                    is.tri = tri;
                    is.mat = mi;
                    is.t = t;
                }
            }
        }
        node = hit ? s->hit_link[face * s->nn + node] : s->miss_link[face * s->nn + node];
        if (node < 0) break;
    }
    if (is.tri >= 0) {
        const vec3 V0 = tri_vertex(s, is.tri, 0), V1 = tri_vertex(s, is.tri, 1), V2 = tri_vertex(s, is.tri, 2);
        const vec3 N0 = tri_normal(s, is.tri, 0), N1 = tri_normal(s, is.tri, 1), N2 = tri_normal(s, is.tri, 2);
        r.t = is.t;
        r.pos = add3(add3(scl3(V2, bu), scl3(V0, bv)), scl3(V1, bw));
        r.nrm = normalize3(add3(add3(scl3(N2, bu), scl3(N0, bv)), scl3(N1, bw)));
        r.texu = (s->tv[is.tri * 3 + 2].w * bu + s->tv[is.tri * 3].w * bv) + s->tv[is.tri * 3 + 1].w * bw;
        r.texv = (s->tn[is.tri * 3 + 2].w * bu + s->tn[is.tri * 3].w * bv) + s->tn[is.tri * 3 + 1].w * bw;
        r.gnrm = normalize3(cross3(sub3(V1, V0), sub3(V2, V0)));
        const vec4 m0 = s->mat[is.mat * 2], m1 = s->mat[is.mat * 2 + 1];
        r.col = xyz(m0);
        r.brdf = (int)m1.x;
        r.g = m1.y;
        r.eta = m0.w;
        r.matid = is.mat;
    }
    *last = is;
    return r;
}

/* ------------------------------------------------------------------------------------------ */
/* BRDF helpers                                                                                */
/* ------------------------------------------------------------------------------------------ */
/* onb (eyeraytrace.fs:293-322 = photontrace.fs:60-89) */
static inline vec3 onb(vec3 x, vec3 n) {
    if (n.z < RC(-0.9999999)) {
        const vec3 u = v3(x.z, x.x, RC(0.0));
        return sub3(lscl3(x.y, n), u);
    }
    const real a = RC(1.0) / (RC(1.0) + n.z);
    const real b = -n.x * n.y * a;
    const vec3 u = v3(RC(1.0) - n.x * n.x * a, b, -n.x);
    const vec3 w = v3(b, RC(1.0) - n.y * n.y * a, -n.y);
    return add3(add3(lscl3(x.x, u), lscl3(x.y, n)), lscl3(x.z, w));
}

/* Fresnel (eyeraytrace.fs:350-367 = photontrace.fs:443-461) */
static inline real fresnel(vec3 incom, vec3 normal, real ii, real ie) {
    const real eta = ii / ie;
    const real c1 = dot3(incom, normal);
    real c2 = RC(1.0) - (eta * eta) * (RC(1.0) - c1 * c1);
    if (c2 < RC(0.0)) return RC(1.0);
    c2 = R_SQRT(c2);
    const real rs = (ii * c1 - ie * c2) / (ii * c1 + ie * c2);
    const real rp = (ii * c2 - ie * c1) / (ii * c2 + ie * c1);
    return (rs * rs + rp * rp) * RC(0.5);
}

/* glossy_reflect (eyeraytrace.fs:370-392 = photontrace.fs:258-280) */
static inline vec3 glossy_reflect(vec3 d, vec3 n, real g, vec4* rndv) {
    const vec3 r = normalize3(add3(lscl3(RC(1.0) - g - g, reflect3(d, n)), lscl3(g + g, n)));
    const real rnd1 = gpu_rnd(rndv);
    const real rnd2 = gpu_rnd(rndv);
    const real temp1 = RC(6.283184) * rnd1;
    const real temp2_ = R_POW(rnd2, g);
    const real temp2 = R_SQRT(RC(1.0) - temp2_ * temp2_);
    const vec3 v = v3(R_SIN(temp1) * temp2, temp2_, R_COS(temp1) * temp2);
    vec3 result = normalize3(onb(v, r));
    if (dot3(result, n) < RC(0.0)) result = reflect3(result, n);
    return result;
}

/* ------------------------------------------------------------------------------------------ */
/* eye pass (eyeraytrace.fs main :396-554)                                                     */
/* ------------------------------------------------------------------------------------------ */
static void eye_pixel(oracle_ctx* c, uint32_t px, uint32_t py) {
    const size_t p = (size_t)py * c->W + px;
    const sppm_camera* cam = &c->cam;
    vec4 rndv = c->q_rng[p];
    const real eps = RC(1e-5);
    const vec3 U = v3(cam->u[0], cam->u[1], cam->u[2]);
    const vec3 V = v3(cam->v[0], cam->v[1], cam->v[2]);
    const vec3 Wd = v3(cam->w[0], cam->w[1], cam->w[2]);
    const vec3 CP = v3(cam->origin[0], cam->origin[1], cam->origin[2]);
    const real cpx = (real)cam->width * RC(0.5), cpy = (real)cam->height * RC(0.5);
    const real fragx = (real)px + RC(0.5), fragy = (real)py + RC(0.5);
    const real ppx = (fragx + c->aa[0]) - cpx;
    const real ppy = (fragy + c->aa[1]) - cpy;
    const vec3 rel = add3(add3(lscl3(ppx, U), lscl3(ppy, V)), lscl3((real)cam->distance, Wd));
    vec3 rdir = normalize3(rel);
    vec3 rorg = CP;
    const real filter = (RC(1.0) - R_FABS(c->aa[0]) / RC(1.5)) * (RC(1.0) - R_FABS(c->aa[1]) / RC(1.5));
    {
        const vec3 fp = add3(CP, scl3(rdir, (real)c->cfg.focal_length));
        const real radius = R_SQRT(gpu_rnd(&rndv)) * (real)c->cfg.aperture;
        const real theta = RC(6.283184) * gpu_rnd(&rndv);
        const vec3 lens = add3(CP, lscl3(radius, add3(scl3(U, R_COS(theta)), scl3(V, R_SIN(theta)))));
        rdir = normalize3(sub3(fp, lens));
        rorg = lens;
    }
    vec3 col = scl3(v3(RC(1.0), RC(1.0), RC(1.0)), filter);
    vec3 nrm = v3(0, 0, 0), pos = v3(0, 0, 0), emi = v3(0, 0, 0);
    LastIsect last = {-1, -1, RC(1.0e20)};
    uint64_t segs = 0;
    for (uint32_t j = 0; j < c->cfg.max_path_length; j++) {
        Isect i = raytrace(c, rorg, rdir, 0, j == 0, &last);
        segs++;
        if (i.t == RC(1.0e+30)) {
            nrm = v3(0, 0, 0);
            if (c->sc.light_area == RC(0.0)) emi = mul3(v3(RC(0.7), RC(0.7), RC(1.0)), col);
            break;
        }
        pos = i.pos;
        nrm = i.nrm;
        if (c->sc.any_tex)
            i.col = tex_modulate(&c->sc, i.texu, i.texv, c->sc.mat_rcp * ((float)i.matid + 0.5f), i.col);
        if (i.brdf == -1) {
            nrm = v3(0, 0, 0);
            emi = mul3(col, i.col);
            break;
        } else if (i.brdf == 0) {
            col = mul3(col, i.col);
            break;
        } else if (i.brdf == 1 || i.brdf == 4) {
            rorg = add3(pos, lscl3(eps, i.gnrm));
            if (i.brdf == 4) nrm = glossy_reflect(nrm, nrm, i.g, &rndv);
            rdir = reflect3(rdir, nrm);
            if (dot3(rdir, i.gnrm) < RC(0.0)) rdir = neg3(rdir);
            col = mul3(col, i.col);
        } else if (i.brdf == 2 || i.brdf == 5) {
            if (i.brdf == 5) nrm = glossy_reflect(nrm, nrm, i.g, &rndv);
            const real ln = dot3(nrm, rdir);
            const real eta = i.eta;
            if (ln < RC(0.0)) {
                const real re = fresnel(neg3(rdir), nrm, RC(1.0), eta);
                if (gpu_rnd(&rndv) < re) {
                    rorg = add3(pos, lscl3(eps, i.gnrm));
                    rdir = reflect3(rdir, nrm);
                    if (dot3(rdir, i.gnrm) < RC(0.0)) rdir = neg3(rdir);
                } else {
                    col = mul3(col, i.col);
                    rorg = sub3(pos, lscl3(eps, i.gnrm));
                    rdir = refract3(rdir, nrm, RC(1.0) / eta);
                    if (dot3(rdir, i.gnrm) > RC(0.0)) rdir = neg3(rdir);
                }
            } else {
                const real re = fresnel(neg3(rdir), neg3(nrm), eta, RC(1.0));
                col = mul3(col, i.col);
                if (gpu_rnd(&rndv) < re) {
                    rorg = sub3(pos, lscl3(eps, i.gnrm));
                    rdir = reflect3(rdir, neg3(nrm));
                    if (dot3(rdir, neg3(i.gnrm)) < RC(0.0)) rdir = neg3(rdir);
                } else {
                    rorg = add3(pos, lscl3(eps, i.gnrm));
                    rdir = refract3(rdir, neg3(nrm), eta);
                    if (dot3(rdir, neg3(i.gnrm)) > RC(0.0)) rdir = neg3(rdir);
                }
            }
        } else if (i.brdf == 3 || i.brdf == 6) {
            if (i.brdf == 6) nrm = glossy_reflect(nrm, nrm, i.g, &rndv);
            const real re = fresnel(neg3(rdir), nrm, RC(1.0), i.eta);
            if (gpu_rnd(&rndv) < re) {
                rorg = add3(pos, lscl3(eps, i.gnrm));
                rdir = reflect3(rdir, nrm);
                if (dot3(rdir, i.gnrm) < RC(0.0)) rdir = neg3(rdir);
            } else {
                col = mul3(col, i.col);
                break;
            }
        }
    }
    vec4 qe = c->q_emi_n[p];
    const real a = RC(1.0) / (real)c->eye_samples;
    qe.x = qe.x * (RC(1.0) - a) + emi.x * a;
    qe.y = qe.y * (RC(1.0) - a) + emi.y * a;
    qe.z = qe.z * (RC(1.0) - a) + emi.z * a;
    c->q_pos[p] = v4(pos, rdir.x);
    c->q_refl[p] = v4(col, rdir.y);
    c->q_nrm[p] = v4(nrm, rdir.z);
    c->q_rng[p] = rndv;
    c->q_tri[p] = last.tri;
    c->q_t[p] = last.t;
    c->q_emi_n[p] = qe;
#pragma omp atomic
    c->eye_segments += segs;
}

/* ------------------------------------------------------------------------------------------ */
/* photon pass (photontrace.fs main :464-720)                                                  */
/* ------------------------------------------------------------------------------------------ */
static void light_sample(oracle_ctx* c, vec4* rndv, vec3* flux, vec3* dir, vec3* org) {
    const oscene* s = &c->sc;
    const real rnd = gpu_rnd(rndv);
    int low = 0;
    int high = (int)(RC(1.0) / s->light_stride + RC(0.5));
    const int nl = (int)s->nl;
    int guard = 0;
    /* texel of the light table at texcoord (mid - 0.5) * stride: nearest, clamped */
#define LIGHT_TEXEL(m)                                                          \
    ({                                                                          \
        real u_ = ((real)(m) - RC(0.5)) * s->light_stride;                      \
        if (u_ < RC(0.0)) u_ = RC(0.0);                                         \
        int k_ = (int)R_FLOOR(u_ * (real)nl);                                   \
        k_ < 0 ? 0 : (k_ > nl - 1 ? nl - 1 : k_);                               \
    })
    while (low < high) {
        if (++guard > 64) {
            c->err = SPPM_ERR_WATCHDOG;
            break;
        }
        const int mid = low + ((high - low) / 2);
        const int k = LIGHT_TEXEL(mid);
        if (s->light_cdf[k] < rnd) low = mid + 1;
        else high = mid;
    }
    const int32_t lt = s->light_tri[LIGHT_TEXEL(high)];
#undef LIGHT_TEXEL
    const real rndv2 = gpu_rnd(rndv);
    const real t = R_SQRT(RC(1.0) - rndv2);
    const real sv = gpu_rnd(rndv);
    const real a = RC(1.0) - t;
    const real cc = sv * t;
    const real b = t - cc;
    const vec3 V0 = tri_vertex(s, lt, 0), V1 = tri_vertex(s, lt, 1), V2 = tri_vertex(s, lt, 2);
    const vec3 N0 = tri_normal(s, lt, 0), N1 = tri_normal(s, lt, 1), N2 = tri_normal(s, lt, 2);
    const int32_t mi = tri_material(s, lt);
    *flux = scl3(xyz(s->mat[mi * 2]), s->light_area * RC(3.141592));
    if (s->any_tex) {
        /* T = T2 * c + T0 * a + T1 * b (photontrace.fs:413-422) */
        const real tu = (s->tv[lt * 3 + 2].w * cc + s->tv[lt * 3].w * a) + s->tv[lt * 3 + 1].w * b;
        const real tw = (s->tn[lt * 3 + 2].w * cc + s->tn[lt * 3].w * a) + s->tn[lt * 3 + 1].w * b;
        *flux = tex_modulate(s, tu, tw, s->mat_rcp * ((float)mi + 0.75f), *flux);
    }
    vec3 o = add3(add3(scl3(V0, a), scl3(V1, b)), scl3(V2, cc));
    const vec3 nrm = normalize3(add3(add3(scl3(N0, a), scl3(N1, b)), scl3(N2, cc)));
    const vec3 gnrm = normalize3(cross3(sub3(V1, V0), sub3(V2, V0)));
    o = add3(o, scl3(gnrm, RC(1.0e-5)));
    real rx = gpu_rnd(rndv);
    real ry = gpu_rnd(rndv);
    rx = RC(6.283184) * rx;
    ry = R_SQRT(ry);
    *dir = onb(v3(R_SIN(rx) * ry, R_SQRT(RC(1.0) - ry * ry), R_COS(rx) * ry), nrm);
    *org = o;
}

static void ibl_sample(oracle_ctx* c, vec4* rndv, vec3* flux, vec3* dir, vec3* org) {
    const real* bs = c->sc.bsphere;
    const real area = RC(12.566368) * bs[3] * bs[3];
    const real temp2 = RC(6.283184) * gpu_rnd(rndv);
    const real aaa = R_SQRT(RC(1.0) - gpu_rnd(rndv));
    const real sinA = R_SIN(aaa);
    const real sinTemp1 = (sinA + sinA) * R_COS(aaa);
    vec3 d = v3(sinTemp1 * R_COS(temp2), RC(1.0) - (sinA + sinA) * sinA, sinTemp1 * R_SIN(temp2));
    if (gpu_rnd(rndv) > RC(0.5)) {
        d = v3(RC(1.0), RC(1.0), RC(1.0));
        d.y += d.y;
        d.z = -d.z;
        d = normalize3(d);
        *flux = scl3(v3(RC(1.0), RC(1.0), RC(0.7)), area);
    } else {
        *flux = scl3(v3(RC(0.7), RC(0.7), RC(1.0)), area);
    }
    const real radius = R_SQRT(gpu_rnd(rndv));
    const real theta = RC(6.283184) * gpu_rnd(rndv);
    const vec3 temp = v3(radius * R_COS(theta), RC(0.0), radius * R_SIN(theta));
    *org = add3(add3(onb(scl3(temp, bs[3]), d), scl3(d, bs[3])), v3(bs[0], bs[1], bs[2]));
    *dir = neg3(d);
}

/* returns 1 when the slot traced a segment this frame */
static int photon_slot(oracle_ctx* c, uint32_t sidx) {
    const oscene* s = &c->sc;
    const real eps = RC(1e-6);
    vec4 rndv = c->p_rng[sidx];
    const vec4 PP = c->p_pos[sidx], PF = c->p_flux[sidx], PD = c->p_dir[sidx];
    const vec3 pnrm = v3(PP.w, PF.w, PD.w);
    vec3 flux = v3(R_FABS(PF.x), R_FABS(PF.y), R_FABS(PF.z));
    vec3 rorg = v3(0, 0, 0), rdir = v3(0, 0, 0);
    int cont;
    uint8_t emitted;
    int32_t ptri = c->frame == 0 ? -1 : c->p_tri[sidx];
    real depth = (c->frame == 0 ? RC(0.0) : (real)c->p_depth[sidx]) + RC(1.0);
    if (ptri < 0 || depth >= (real)c->cfg.max_path_length) {
        if (s->light_area != RC(0.0)) light_sample(c, &rndv, &flux, &rdir, &rorg);
        else ibl_sample(c, &rndv, &flux, &rdir, &rorg);
        emitted = 1;
        depth = RC(0.0);
        cont = 1;
    } else {
        const vec3 V0 = tri_vertex(s, ptri, 0), V1 = tri_vertex(s, ptri, 1), V2 = tri_vertex(s, ptri, 2);
        const vec3 gnrm = normalize3(cross3(sub3(V1, V0), sub3(V2, V0)));
        const vec3 ipos = xyz(PP);
        vec3 inrm = pnrm;
        const int32_t mi = tri_material(s, ptri);
        vec3 icol = xyz(s->mat[mi * 2]);
        if (s->any_tex) {
            /* the hit's barycentrics from the stored position (photontrace.fs:521-545) */
            const real bx = len3(cross3(sub3(V1, V0), sub3(ipos, V0)));
            const real by = len3(cross3(sub3(V2, V1), sub3(ipos, V1)));
            const real bz = len3(cross3(sub3(V0, V2), sub3(ipos, V2)));
            const real bw_ = (bx + by) + bz;
            const real nx = bx / bw_, ny = by / bw_, nz = bz / bw_;
            const real tu = (s->tv[ptri * 3 + 2].w * nx + s->tv[ptri * 3].w * ny) + s->tv[ptri * 3 + 1].w * nz;
            const real tw = (s->tn[ptri * 3 + 2].w * nx + s->tn[ptri * 3].w * ny) + s->tn[ptri * 3 + 1].w * nz;
            icol = tex_modulate(s, tu, tw, s->mat_rcp * (((float)mi + 0.5f) + 0.25f), icol);
        }
        const int brdf = (int)s->mat[mi * 2 + 1].x;
        const real ieta = s->mat[mi * 2].w;
        const real ig = s->mat[mi * 2 + 1].y;
        const vec3 pd = xyz(PD);
        if (brdf == 0) {
            const real r0 = RC(6.283184) * gpu_rnd(&rndv);
            const real r1 = R_SQRT(gpu_rnd(&rndv));
            const vec3 v = v3(R_SIN(r0) * r1, R_SQRT(RC(1.0) - r1 * r1), R_COS(r0) * r1);
            rorg = add3(ipos, lscl3(eps, gnrm));
            rdir = onb(v, inrm);
            if (dot3(rdir, gnrm) < RC(0.0)) rdir = neg3(rdir);
        } else if (brdf == 1 || brdf == 4) {
            rorg = add3(ipos, lscl3(eps, gnrm));
            if (brdf == 4) inrm = glossy_reflect(inrm, inrm, ig, &rndv);
            rdir = reflect3(pd, inrm);
            if (dot3(rdir, gnrm) < RC(0.0)) rdir = neg3(rdir);
        } else if (brdf == 2 || brdf == 5) {
            if (brdf == 5) inrm = glossy_reflect(inrm, inrm, ig, &rndv);
            const real ln = dot3(inrm, pd);
            if (ln < RC(0.0)) {
                const real re = fresnel(neg3(pd), inrm, RC(1.0), ieta);
                if (gpu_rnd(&rndv) < re) {
                    rorg = add3(ipos, lscl3(eps, gnrm));
                    rdir = reflect3(pd, inrm);
                    icol = v3(RC(1.0), RC(1.0), RC(1.0));
                    if (dot3(rdir, gnrm) < RC(0.0)) rdir = neg3(rdir);
                } else {
                    rorg = sub3(ipos, lscl3(eps, gnrm));
                    rdir = refract3(pd, inrm, RC(1.0) / ieta);
                    if (dot3(rdir, gnrm) > RC(0.0)) rdir = neg3(rdir);
                }
            } else {
                const real re = fresnel(neg3(pd), neg3(inrm), ieta, RC(1.0));
                if (gpu_rnd(&rndv) < re) {
                    rorg = sub3(ipos, lscl3(eps, gnrm));
                    rdir = reflect3(pd, neg3(inrm));
                    if (dot3(rdir, neg3(gnrm)) < RC(0.0)) rdir = neg3(rdir);
                } else {
                    rorg = add3(ipos, lscl3(eps, gnrm));
                    rdir = refract3(pd, neg3(inrm), ieta);
                    if (dot3(rdir, neg3(gnrm)) > RC(0.0)) rdir = neg3(rdir);
                }
            }
        } else if (brdf == 3 || brdf == 6) {
            if (brdf == 6) inrm = glossy_reflect(inrm, inrm, ig, &rndv);
            const real re = fresnel(neg3(pd), inrm, RC(1.0), ieta);
            if (gpu_rnd(&rndv) < re) {
                rorg = add3(ipos, lscl3(eps, gnrm));
                rdir = reflect3(pd, inrm);
                icol = v3(RC(1.0), RC(1.0), RC(1.0));
                if (dot3(rdir, gnrm) < RC(0.0)) rdir = neg3(rdir);
            } else {
                const real r0 = RC(6.283184) * gpu_rnd(&rndv);
                const real r1 = R_SQRT(gpu_rnd(&rndv));
                const vec3 v = v3(R_SIN(r0) * r1, R_SQRT(RC(1.0) - r1 * r1), R_COS(r0) * r1);
                rorg = add3(ipos, lscl3(eps, gnrm));
                rdir = onb(v, inrm);
                if (dot3(rdir, gnrm) < RC(0.0)) rdir = neg3(rdir);
            }
        }
        /* Russian roulette (:671-685) */
        const real pmax = R_FMAX(R_FMAX(icol.x, icol.y), icol.z);
        if (pmax < gpu_rnd(&rndv)) {
            cont = 0;
        } else {
            cont = 1;
            icol = v3(icol.x / pmax, icol.y / pmax, icol.z / pmax);
            flux = mul3(flux, icol);
        }
        emitted = 0;
    }
    if (cont) {
        LastIsect last;
        const Isect i = raytrace(c, rorg, rdir, 1, 0, &last);
        if (i.t == RC(1.0e+30) || (i.brdf != 0 && i.brdf != 6 && i.brdf != 3)) flux = neg3(flux);
        const real gf = R_FMIN(R_FABS(dot3(rdir, i.nrm) / dot3(rdir, i.gnrm)), R_SQRT(RC(5.0)));
        flux = scl3(flux, gf);
        c->p_pos[sidx] = v4(i.pos, i.nrm.x);
        c->p_flux[sidx] = v4(flux, i.nrm.y);
        c->p_dir[sidx] = v4(rdir, i.nrm.z);
        c->p_rng[sidx] = rndv;
        c->p_tri[sidx] = last.tri;
        c->p_depth[sidx] = (int32_t)depth;
        c->p_t[sidx] = last.t;
    } else {
        c->p_pos[sidx] = v4(v3(0, 0, 0), RC(0.0));
        c->p_flux[sidx] = v4(v3(RC(-1.0), RC(-1.0), RC(-1.0)), RC(0.0));
        c->p_dir[sidx] = v4(v3(0, 0, 0), RC(0.0));
        c->p_rng[sidx] = rndv;
        c->p_tri[sidx] = -1;
        c->p_depth[sidx] = 0;
        c->p_t[sidx] = RC(1e+30);
    }
    c->p_emitted[sidx] = emitted;
    return cont;
}

/* ------------------------------------------------------------------------------------------ */
/* stochastic hashed grid (hash.fs, scatter.vs + GL_LESS depth test, correction.vs + blend)   */
/* ------------------------------------------------------------------------------------------ */
static void hash_build(oracle_ctx* c) {
    const real hs1 = RC(4194304.0) / c->grid_scale;
    const real hn = (real)c->hash_num;
    for (uint32_t k = 0; k < c->hash_num; k++) {
        c->winner[k] = 0xFFFFFFFFu;
        c->count[k] = 0;
    }
    const real pb1 = RC(1.0) / (real)c->PH; /* PhotonBufferSize1 */
    for (uint32_t j = 0; j < c->PH; j++) {
        for (uint32_t i = 0; i < c->PW; i++) {
            const uint32_t id = j * c->PW + i;
            if (c->p_flux[id].x < RC(0.0)) continue; /* invalid photon: slot -1, clipped */
            const vec3 pp = xyz(c->p_pos[id]);
            const vec3 cell = v3(R_FLOOR((pp.x - c->bbmin[0]) * c->grid_scale),
                                 R_FLOOR((pp.y - c->bbmin[1]) * c->grid_scale),
                                 R_FLOOR((pp.z - c->bbmin[2]) * c->grid_scale));
            const uint32_t slot = hash_cell(cell, c->grid_scale, hs1, hn);
            c->count[slot] += 1; /* correction.vs: additive blend of 1.0 */
            /* scatter.vs: z = s * (1/P) + t with (s, t) the photon's texel centre */
            const real sx = ((real)i + RC(0.5)) / (real)c->PW;
            const real ty = ((real)j + RC(0.5)) / (real)c->PH;
            const real z = sx * pb1 + ty;
            if (!(c->cfg.flags & SPPM_FLAG_GL_DEPTH_CLIP) || z < RC(1.0)) {
                if (id < c->winner[slot]) c->winner[slot] = id; /* GL_LESS keeps the nearest */
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* progressive.fs                                                                              */
/* ------------------------------------------------------------------------------------------ */
static void gather_pixel(oracle_ctx* c, size_t p) {
    const real G = c->grid_scale;
    const real hs1 = RC(4194304.0) / G;
    const real hn = (real)c->hash_num;
    const real alpha = (real)c->cfg.alpha;
    const vec3 qp = xyz(c->q_pos[p]), qn = xyz(c->q_nrm[p]);
    vec4 qfr = c->q_flux_r[p];
    vec4 qe = c->q_emi_n[p];
    const vec3 qr = xyz(c->q_refl[p]);
    real N = qe.w;
    real R = qfr.w;
    vec3 tau = xyz(qfr);
    if (c->q_tri[p] >= 0) {
        const vec3 ii = v3(R_FLOOR(R_FABS(qp.x - c->bbmin[0]) * G - RC(0.5)),
                           R_FLOOR(R_FABS(qp.y - c->bbmin[1]) * G - RC(0.5)),
                           R_FLOOR(R_FABS(qp.z - c->bbmin[2]) * G - RC(0.5)));
        vec3 flux = v3(0, 0, 0);
        real M = RC(0.0);
        for (int iz = 0; iz <= 1; iz++) {
            for (int iy = 0; iy <= 1; iy++) {
                for (int ix = 0; ix <= 1; ix++) {
                    const vec3 cell = add3(ii, v3((real)ix, (real)iy, (real)iz));
                    const uint32_t slot = hash_cell(cell, G, hs1, hn);
                    /* an empty slot reads the cleared texel (0,0): photon 0 with count 0 */
                    const uint32_t w = c->winner[slot] == 0xFFFFFFFFu ? 0u : c->winner[slot];
                    const vec4 pf = c->p_flux[w], pp = c->p_pos[w], pd = c->p_dir[w];
                    const vec3 rmin = v3(cell.x / G + c->bbmin[0], cell.y / G + c->bbmin[1], cell.z / G + c->bbmin[2]);
                    const vec3 rmax = v3((cell.x + RC(1.0)) / G + c->bbmin[0], (cell.y + RC(1.0)) / G + c->bbmin[1],
                                         (cell.z + RC(1.0)) / G + c->bbmin[2]);
                    if (pp.x > rmin.x && pp.y > rmin.y && pp.z > rmin.z && pp.x < rmax.x && pp.y < rmax.y &&
                        pp.z < rmax.z) {
                        const vec3 diff = sub3(xyz(pp), qp);
                        if (length3(diff) < R && dot3(qn, neg3(xyz(pd))) > RC(0.0)) {
                            const real cnt = (real)c->count[slot];
                            flux = add3(flux, scl3(xyz(pf), cnt));
                            M += cnt;
                        }
                    }
                }
            }
        }
        flux = mul3(flux, scl3(qr, RC(0.31830995240629591621063460818591)));
        const real g = R_FMIN((N + alpha * M) / (N + M), RC(1.0));
        R = R * R_SQRT(g);
        N = N + M * alpha;
        tau = scl3(add3(tau, flux), g);
    }
    c->q_flux_r[p] = v4(tau, R);
    qe.w = N;
    c->q_emi_n[p] = qe;
}

/* ------------------------------------------------------------------------------------------ */
/* counting-sort photon grid (SPPM_FLAG_PHOTON_GRID) -- not part of the reference: the CUDA      */
/* mixed path's estimator, which keeps every stored photon sorted by the reference's hash slot  */
/* (hash.fs:51-68) and sums all photons of the 2x2x2 cells inside the radius (progressive.fs's   */
/* AccumulatePhotons :65-95 over every photon instead of a slot's winner times its count).      */
/* The single-precision build restates the CUDA records bit for bit (21-bit grid fixed point,   */
/* FP16 flux scaled by 1/(light area * 3.141592), 8-bit octahedral direction; the CUDA side is  */
/* glslppm_gb300/csrc/cuda/photon_grid.cuh), so it counts the same photons per pixel and forms  */
/* the same flux sums; the double-precision build gathers the unquantised photons.              */
/* ------------------------------------------------------------------------------------------ */
static uint32_t grid_photon_slot(const oracle_ctx* c, uint32_t id) {
    const real hs1 = RC(4194304.0) / c->grid_scale;
    const vec3 pp = xyz(c->p_pos[id]);
    const vec3 cell = v3(R_FLOOR((pp.x - c->bbmin[0]) * c->grid_scale), R_FLOOR((pp.y - c->bbmin[1]) * c->grid_scale),
                         R_FLOOR((pp.z - c->bbmin[2]) * c->grid_scale));
    return hash_cell(cell, c->grid_scale, hs1, (real)c->hash_num);
}

/* the stored photons (flux >= 0) by slot, ids ascending within a slot */
static void grid_build(oracle_ctx* c) {
    memset(c->g_ofs, 0, sizeof(uint32_t) * ((size_t)c->hash_num + 1));
    for (uint32_t id = 0; id < c->P; id++)
        if (c->p_flux[id].x >= RC(0.0)) c->g_ofs[grid_photon_slot(c, id) + 1]++;
    for (uint32_t k = 0; k < c->hash_num; k++) c->g_ofs[k + 1] += c->g_ofs[k];
    memcpy(c->g_cur, c->g_ofs, sizeof(uint32_t) * c->hash_num);
    for (uint32_t id = 0; id < c->P; id++)
        if (c->p_flux[id].x >= RC(0.0)) c->g_ids[c->g_cur[grid_photon_slot(c, id)]++] = id;
}

#ifndef ORACLE_FP64
static int grid_frac_bits(const oracle_ctx* c) {
    uint32_t cells = 0;
    for (int k = 0; k < 3; k++) {
        const float e = (c->bbmax[k] - c->bbmin[k]) * c->grid_scale;
        const uint32_t n = e > 0.0f ? (e < 2097152.0f ? (uint32_t)ceilf(e) : 2097152u) : 0u;
        if (n > cells) cells = n;
    }
    int b = 0;
    for (uint32_t v = cells + 1u; v; v >>= 1) b++;
    return b < 21 ? 21 - b : 0;
}
static uint32_t grid_coord(float p, float bbmin, float G, float sF) {
    const float v = ((p - bbmin) * G) * sF;
    return v >= 0.0f && v < 2097151.0f ? (uint32_t)v : 0x1FFFFFu;
}
/* IEEE round-to-nearest-even conversion of a non-negative float of at most 65504 to FP16 bits */
static uint32_t half_rn(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    const uint32_t e = (x >> 23) & 0xFFu, m = x & 0x7FFFFFu;
    if (e == 0) return 0u;
    const int he = (int)e - 112; /* FP16 biased exponent */
    if (he <= 0) {               /* FP16 subnormal: the value in units of 2^-24 is (m | 2^23) / 2^(126 - e) */
        const uint32_t s = 126u - e, mf = m | 0x800000u;
        if (s > 24u) return 0u;
        const uint32_t q = mf >> s, rem = mf & ((1u << s) - 1u), half = 1u << (s - 1u);
        return q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
    }
    uint32_t h = ((uint32_t)he << 10) | (m >> 13);
    const uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return h;
}
static uint32_t grid_oct8(float x, float y, float z) {
    const float s = (fabsf(x) + fabsf(y)) + fabsf(z);
    if (!(s > 0.0f)) return 0u;
    float ox = x / s, oy = y / s;
    if (z < 0.0f) {
        const float tx = (1.0f - fabsf(oy)) * copysignf(1.0f, ox);
        const float ty = (1.0f - fabsf(ox)) * copysignf(1.0f, oy);
        ox = tx;
        oy = ty;
    }
    const int a = (int)lrintf(ox * 127.0f), b = (int)lrintf(oy * 127.0f);
    return ((uint32_t)a & 0xFFu) | (((uint32_t)b & 0xFFu) << 8);
}
static float grid_oct8_dot(uint32_t code, float nx, float ny, float nz) {
    float x = (float)(int)(int8_t)(code & 0xFFu), y = (float)(int)(int8_t)((code >> 8) & 0xFFu);
    const float ax = fabsf(x), ay = fabsf(y);
    const float z = 127.0f - ax - ay;
    if (z < 0.0f) {
        const float tx = (127.0f - ay) * copysignf(1.0f, x);
        y = (127.0f - ax) * copysignf(1.0f, y);
        x = tx;
    }
    return (nx * x + ny * y) + nz * z;
}
static uint64_t half_fixed(uint32_t h) {
    const uint32_t e = (h >> 10) & 31u, m = h & 1023u;
    return e ? (uint64_t)(m | 1024u) << (e - 1u) : (uint64_t)m;
}
#endif

static void grid_gather_pixel(oracle_ctx* c, size_t p) {
    const real G = c->grid_scale;
    const real hs1 = RC(4194304.0) / G;
    const real hn = (real)c->hash_num;
    const real alpha = (real)c->cfg.alpha;
    const vec3 qp = xyz(c->q_pos[p]), qn = xyz(c->q_nrm[p]);
    vec4 qfr = c->q_flux_r[p];
    vec4 qe = c->q_emi_n[p];
    const vec3 qr = xyz(c->q_refl[p]);
    real N = qe.w;
    real R = qfr.w;
    vec3 tau = xyz(qfr);
    if (c->q_tri[p] >= 0) {
        const real gx = R_FABS(qp.x - c->bbmin[0]) * G, gy = R_FABS(qp.y - c->bbmin[1]) * G,
                   gz = R_FABS(qp.z - c->bbmin[2]) * G;
        vec3 flux = v3(0, 0, 0);
        real M = RC(0.0);
        /* the reference cells the sphere of radius R touches (every photon inside R is in one) */
#ifndef ORACLE_FP64
        const int F = grid_frac_bits(c);
        const float sF = ldexpf(1.0f, F);
        const float ux = gx * sF, uy = gy * sF, uz = gz * sF;
        const float rq2 = ((R * R * G) * G) * (sF * sF);
        const float rq = sqrtf(rq2) * 1.0001f + 1.0f;
        const float fu = c->sc.light_area != 0.0f ? c->sc.light_area * 3.141592f : 1.0f, fs = 1.0f / fu;
        uint64_t sr = 0, sg = 0, sb = 0;
        uint32_t m = 0;
#define GRID_LO(u) ((u) - rq > 0.0f ? (int)((uint32_t)((u) - rq) >> F) : 0)
#define GRID_HI(u) ((int)(((u) + rq < 2097150.0f ? (uint32_t)((u) + rq) : 2097150u) >> F))
        const int x0 = GRID_LO(ux), x1 = GRID_HI(ux), y0 = GRID_LO(uy), y1 = GRID_HI(uy), z0 = GRID_LO(uz),
                  z1 = GRID_HI(uz);
#undef GRID_LO
#undef GRID_HI
#else
        const real rg = R * G * (1.0 + 1e-9);
        const int x0 = (int)floor(gx - rg), x1 = (int)floor(gx + rg), y0 = (int)floor(gy - rg), y1 = (int)floor(gy + rg),
                  z0 = (int)floor(gz - rg), z1 = (int)floor(gz + rg);
#endif
        for (int iz = z0; iz <= z1; iz++) {
            for (int iy = y0; iy <= y1; iy++) {
                for (int ix = x0; ix <= x1; ix++) {
                    const vec3 cell = v3((real)ix, (real)iy, (real)iz);
                    const uint32_t slot = hash_cell(cell, G, hs1, hn);
                    for (uint32_t k = c->g_ofs[slot]; k < c->g_ofs[slot + 1]; k++) {
                        const uint32_t id = c->g_ids[k];
                        const vec4 pf = c->p_flux[id], pp = c->p_pos[id], pd = c->p_dir[id];
#ifndef ORACLE_FP64
                        const uint32_t qx = grid_coord(pp.x, c->bbmin[0], G, sF), qy = grid_coord(pp.y, c->bbmin[1], G, sF),
                                       qz = grid_coord(pp.z, c->bbmin[2], G, sF);
                        if ((qx >> F) != (uint32_t)cell.x || (qy >> F) != (uint32_t)cell.y || (qz >> F) != (uint32_t)cell.z)
                            continue;
                        const float dx = ((float)qx + 0.5f) - ux, dy = ((float)qy + 0.5f) - uy, dz = ((float)qz + 0.5f) - uz;
                        if (!((dx * dx + dy * dy) + dz * dz < rq2)) continue;
                        if (!(grid_oct8_dot(grid_oct8(pd.x, pd.y, pd.z), qn.x, qn.y, qn.z) < 0.0f)) continue;
                        sr += half_fixed(half_rn(fminf(pf.x * fs, 65504.0f)));
                        sg += half_fixed(half_rn(fminf(pf.y * fs, 65504.0f)));
                        sb += half_fixed(half_rn(fminf(pf.z * fs, 65504.0f)));
                        m++;
#else
                        const vec3 pc = v3(R_FLOOR((pp.x - c->bbmin[0]) * G), R_FLOOR((pp.y - c->bbmin[1]) * G),
                                           R_FLOOR((pp.z - c->bbmin[2]) * G));
                        if (pc.x != cell.x || pc.y != cell.y || pc.z != cell.z) continue;
                        if (!(length3(sub3(xyz(pp), qp)) < R && dot3(qn, neg3(xyz(pd))) > RC(0.0))) continue;
                        flux = add3(flux, xyz(pf));
                        M += RC(1.0);
#endif
                    }
                }
            }
        }
#ifndef ORACLE_FP64
        flux = v3(((float)sr * 5.9604644775390625e-8f) * fu, ((float)sg * 5.9604644775390625e-8f) * fu,
                  ((float)sb * 5.9604644775390625e-8f) * fu);
        M = (float)m;
#endif
        flux = mul3(flux, scl3(qr, RC(0.31830995240629591621063460818591)));
        const real g = R_FMIN((N + alpha * M) / (N + M), RC(1.0));
        R = R * R_SQRT(g);
        N = N + M * alpha;
        tau = scl3(add3(tau, flux), g);
    }
    c->q_flux_r[p] = v4(tau, R);
    qe.w = N;
    c->q_emi_n[p] = qe;
}

/* ------------------------------------------------------------------------------------------ */
/* frame schedule (m_display, glslppm.cpp:214-536)                                             */
/* ------------------------------------------------------------------------------------------ */
static float xorshift_frand(uint32_t* s) {
    const uint32_t t = s[0] ^ (s[0] << 11);
    s[0] = s[1];
    s[1] = s[2];
    s[2] = s[3];
    s[3] = (s[3] ^ (s[3] >> 19)) ^ (t ^ (t >> 8));
    return (float)s[3] * (1.0f / 4294967295.0f);
}

static uint32_t mix32(uint32_t h) { /* MurmurHash3 fmix32 finaliser */
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

static void seed_state(oracle_ctx* c) {
    c->xs[0] = 123456789u;
    c->xs[1] = 362436069u;
    c->xs[2] = 521288629u;
    c->xs[3] = 88675123u;
    if (c->cfg.seed != 0) {
        for (int k = 0; k < 4; k++) c->xs[k] ^= mix32(c->cfg.seed * 4u + (uint32_t)k + 0x9E3779B9u);
        if ((c->xs[0] | c->xs[1] | c->xs[2] | c->xs[3]) == 0) c->xs[0] = 1;
    }
    const size_t npix = (size_t)c->W * c->H;
    if (c->cfg.seed_mode == SPPM_SEED_XORSHIFT) {
        for (size_t p = 0; p < npix; p++) {
            float v[4];
            for (int k = 3; k >= 0; k--) v[k] = (float)((double)xorshift_frand(c->xs) * 4194304.0);
            c->q_rng[p].x = v[0];
            c->q_rng[p].y = v[1];
            c->q_rng[p].z = v[2];
            c->q_rng[p].w = v[3];
        }
        for (size_t p = 0; p < c->P; p++) {
            float v[4];
            for (int k = 3; k >= 0; k--) v[k] = (float)((double)xorshift_frand(c->xs) * 4194304.0);
            c->p_rng[p].x = v[0];
            c->p_rng[p].y = v[1];
            c->p_rng[p].z = v[2];
            c->p_rng[p].w = v[3];
        }
    } else {
        /* lane k of element e: an integer state in [1, m_k - 1] from a hash of (seed, e, k) */
        static const uint32_t mlane[4] = {4194287u, 4194277u, 4194191u, 4194167u};
        for (size_t e = 0; e < npix + c->P; e++) {
            real v[4];
            for (int k = 0; k < 4; k++) {
                const uint32_t h = mix32(mix32((uint32_t)e * 4u + (uint32_t)k) ^ mix32(c->cfg.seed + 0x51ED27u * (e >= npix)));
                v[k] = (real)(1u + h % (mlane[k] - 1u));
            }
            vec4* dst = e < npix ? &c->q_rng[e] : &c->p_rng[e - npix];
            dst->x = v[0];
            dst->y = v[1];
            dst->z = v[2];
            dst->w = v[3];
        }
    }
}

static void reset_state(oracle_ctx* c) {
    const size_t npix = (size_t)c->W * c->H;
    memset(c->q_pos, 0, sizeof(vec4) * npix);
    memset(c->q_refl, 0, sizeof(vec4) * npix);
    memset(c->q_nrm, 0, sizeof(vec4) * npix);
    memset(c->q_emi_n, 0, sizeof(vec4) * npix);
    memset(c->q_flux_r, 0, sizeof(vec4) * npix);
    for (size_t p = 0; p < npix; p++) {
        c->q_tri[p] = -1;
        c->q_t[p] = RC(1.0e20);
    }
    memset(c->p_pos, 0, sizeof(vec4) * c->P);
    memset(c->p_flux, 0, sizeof(vec4) * c->P);
    memset(c->p_dir, 0, sizeof(vec4) * c->P);
    for (size_t p = 0; p < c->P; p++) {
        c->p_tri[p] = -1;
        c->p_depth[p] = 0;
        c->p_t[p] = RC(1e30);
        c->p_emitted[p] = 0;
    }
    for (uint32_t k = 0; k < c->hash_num; k++) {
        c->winner[k] = 0xFFFFFFFFu;
        c->count[k] = 0;
    }
    c->frame = 0;
    c->eye_samples = 0;
    c->num_photons = 0;
    c->num_photons_f32 = 0.0f;
    c->photon_segments = c->eye_segments = 0;
    c->initial_radius = c->grid_scale = RC(0.0);
    c->err = 0;
    seed_state(c);
}

static void run_frame(oracle_ctx* c) {
    const size_t npix = (size_t)c->W * c->H;
    const uint32_t interval = c->cfg.eye_pass_interval ? c->cfg.eye_pass_interval : 1;
    if (c->frame % interval == 0) {
        c->aa[0] = (real)((xorshift_frand(c->xs) - 0.5f) * 1.25f);
        c->aa[1] = (real)((xorshift_frand(c->xs) - 0.5f) * 1.25f);
        c->eye_samples++;
#pragma omp parallel for schedule(dynamic, 16)
        for (long long py = 0; py < (long long)c->H; py++)
            for (uint32_t px = 0; px < c->W; px++) eye_pixel(c, px, (uint32_t)py);
        /* ReduceTexture(max), ReduceTexture(min) over QueryPositionTexture */
        real mx[3] = {c->q_pos[0].x, c->q_pos[0].y, c->q_pos[0].z};
        real mn[3] = {mx[0], mx[1], mx[2]};
        for (size_t p = 1; p < npix; p++) {
            const real v[3] = {c->q_pos[p].x, c->q_pos[p].y, c->q_pos[p].z};
            for (int k = 0; k < 3; k++) {
                mx[k] = R_FMAX(mx[k], v[k]);
                mn[k] = R_FMIN(mn[k], v[k]);
            }
        }
        real r0;
        if (c->cfg.radius_rule == SPPM_RADIUS_DIAGONAL) {
            r0 = c->initial_radius; /* fixed at create time */
        } else {
            real bbsize = RC(0.0);
            for (int k = 0; k < 3; k++) bbsize += mx[k] - mn[k];
            r0 = (bbsize / RC(3.0)) / (real)c->W * (real)c->cfg.initial_footprint;
        }
        c->initial_radius = r0;
        for (int k = 0; k < 3; k++) {
            c->bbmin[k] = mn[k] - r0;
            c->bbmax[k] = mx[k] + r0;
        }
        c->grid_scale = RC(0.5) / r0;
    }
    if (c->frame == 0) {
        for (size_t p = 0; p < npix; p++) {
            c->q_flux_r[p].x = c->q_flux_r[p].y = c->q_flux_r[p].z = RC(0.0);
            c->q_flux_r[p].w = c->initial_radius;
        }
        c->num_photons = 0;
        c->num_photons_f32 = 0.0f;
    }
    uint64_t emitted = 0, segments = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : emitted, segments)
    for (long long sidx = 0; sidx < (long long)c->P; sidx++) {
        segments += (uint64_t)photon_slot(c, (uint32_t)sidx);
        emitted += c->p_emitted[sidx];
    }
    c->photon_segments += segments;
    c->num_photons += emitted;
    c->num_photons_f32 += (float)(int)emitted;
    if (c->cfg.flags & SPPM_FLAG_PHOTON_GRID) {
        grid_build(c);
#pragma omp parallel for schedule(dynamic, 256)
        for (long long p = 0; p < (long long)npix; p++) grid_gather_pixel(c, (size_t)p);
    } else {
        hash_build(c);
#pragma omp parallel for schedule(static)
        for (long long p = 0; p < (long long)npix; p++) gather_pixel(c, (size_t)p);
    }
    c->frame++;
}

/* ------------------------------------------------------------------------------------------ */
/* exported entry points                                                                       */
/* ------------------------------------------------------------------------------------------ */
EXPORT void ORACLE_API(destroy)(oracle_ctx* c);

EXPORT oracle_ctx* ORACLE_API(create)(const sppm_config* cfg, const sppm_scene* scene, const sppm_camera* cam) {
    rnd_init_constants();
    if (!cfg || !scene || !cam || scene->num_nodes != 2 * scene->num_triangles - 1) return NULL;
    oracle_ctx* c = (oracle_ctx*)calloc(1, sizeof(oracle_ctx));
    c->cfg = *cfg;
    c->cam = *cam;
    c->W = cfg->width;
    c->H = cfg->height;
    c->PW = cfg->photon_width;
    c->PH = cfg->photon_height;
    c->P = c->PW * c->PH;
    c->hash_num = cfg->hash_slots ? cfg->hash_slots : c->P;
    oscene* s = &c->sc;
    const uint32_t nt = scene->num_triangles, nn = scene->num_nodes;
    s->nt = nt;
    s->nm = scene->num_materials;
    s->nl = scene->num_lights;
    s->nn = nn;
    s->tv = (vec4*)malloc(sizeof(vec4) * nt * 3);
    s->tn = (vec4*)malloc(sizeof(vec4) * nt * 3);
    for (uint32_t t = 0; t < nt; t++) {
        for (int k = 0; k < 3; k++) {
            const float* p = &scene->positions[t * 9 + k * 3];
            const float* n = &scene->normals[t * 9 + k * 3];
            const float tu = scene->texcoords ? scene->texcoords[t * 6 + k * 2] : 1.0e30f;
            const float tw = scene->texcoords ? scene->texcoords[t * 6 + k * 2 + 1] : 1.0e30f;
            const float sg = n[2] > 0.0f ? 1.0f : -1.0f; /* sgn() of gpurt.cpp:35-45 */
            s->tv[t * 3 + k].x = p[0];
            s->tv[t * 3 + k].y = p[1];
            s->tv[t * 3 + k].z = p[2];
            s->tv[t * 3 + k].w = tu;
            s->tn[t * 3 + k].x = n[0];
            s->tn[t * 3 + k].y = n[1];
            s->tn[t * 3 + k].z = sg * (float)(scene->material_ids[t] + 1);
            s->tn[t * 3 + k].w = tw;
        }
    }
    s->mat = (vec4*)malloc(sizeof(vec4) * s->nm * 2);
    for (uint32_t m = 0; m < s->nm; m++) {
        const sppm_material* mm = &scene->materials[m];
        s->mat[m * 2].x = mm->color[0];
        s->mat[m * 2].y = mm->color[1];
        s->mat[m * 2].z = mm->color[2];
        s->mat[m * 2].w = mm->eta;
        s->mat[m * 2 + 1].x = (real)mm->brdf;
        s->mat[m * 2 + 1].y = mm->glossiness;
        s->mat[m * 2 + 1].z = 0;
        s->mat[m * 2 + 1].w = 0;
    }
    s->light_tri = (int32_t*)malloc(sizeof(int32_t) * (s->nl + 1));
    s->light_cdf = (real*)malloc(sizeof(real) * (s->nl + 1));
    for (uint32_t l = 0; l < s->nl; l++) {
        s->light_tri[l] = scene->light_triangles[l];
        s->light_cdf[l] = scene->light_cdf[l];
    }
    s->light_area = scene->light_area;
    s->light_stride = s->nl ? (real)(1.0f / (float)s->nl) : RC(0.0);
    s->mat_rcp = 1.0f / (float)s->nm;
    s->mat_layer = (int32_t*)malloc(sizeof(int32_t) * s->nm);
    for (uint32_t m = 0; m < s->nm; m++)
        s->mat_layer[m] = (scene->num_textures && scene->material_texture) ? scene->material_texture[m] : -1;
    s->any_tex = 0;
    if (scene->texcoords)
        for (size_t k = 0; k < (size_t)nt * 6; k++)
            if (fabsf(scene->texcoords[k]) < 1e10f) s->any_tex = 1;
    s->tex = NULL;
    if (scene->num_textures && scene->textures && scene->material_texture) {
        const size_t bytes = (size_t)scene->num_textures * SPPM_TEXTURE_RES * SPPM_TEXTURE_RES * 4;
        s->tex = (uint8_t*)malloc(bytes);
        memcpy(s->tex, scene->textures, bytes);
    }
    {
        /* SceneBSphere (glslppm.cpp:388-393) in single precision on the host */
        const float* mn = scene->bbox_min;
        const float* mx = scene->bbox_max;
        const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        s->bsphere[0] = (mx[0] + mn[0]) * 0.5f;
        s->bsphere[1] = (mx[1] + mn[1]) * 0.5f;
        s->bsphere[2] = (mx[2] + mn[2]) * 0.5f;
        s->bsphere[3] = sqrtf(dx * dx + dy * dy + dz * dz) * 0.5f;
    }
    s->nb = (real*)malloc(sizeof(real) * nn * 6);
    s->ntri = (int32_t*)malloc(sizeof(int32_t) * nn);
    for (uint32_t i = 0; i < nn * 6; i++) s->nb[i] = scene->node_bounds[i];
    for (uint32_t i = 0; i < nn; i++) s->ntri[i] = scene->node_triangle[i];
    /* hit/miss links of each ordering in canonical numbering (gpurt.cpp:332-366, 415-470) */
    s->hit_link = (int32_t*)malloc(sizeof(int32_t) * nn * 6);
    s->miss_link = (int32_t*)malloc(sizeof(int32_t) * nn * 6);
    for (int o = 0; o < 6; o++) {
        const int32_t* base = &scene->order_base[(size_t)o * nn];
        const int32_t* miss = &scene->order_miss[(size_t)o * nn];
        for (uint32_t i = 0; i < nn; i++) {
            const int32_t cid = base[i];
            s->hit_link[o * nn + cid] = (i + 1 >= nn) ? -1 : base[i + 1];
            s->miss_link[o * nn + cid] = (miss[i] == -1 || miss[i] >= (int32_t)nn) ? -1 : base[miss[i]];
        }
    }
    const size_t npix = (size_t)c->W * c->H;
    c->q_pos = (vec4*)malloc(sizeof(vec4) * npix);
    c->q_refl = (vec4*)malloc(sizeof(vec4) * npix);
    c->q_nrm = (vec4*)malloc(sizeof(vec4) * npix);
    c->q_rng = (vec4*)malloc(sizeof(vec4) * npix);
    c->q_emi_n = (vec4*)malloc(sizeof(vec4) * npix);
    c->q_flux_r = (vec4*)malloc(sizeof(vec4) * npix);
    c->q_tri = (int32_t*)malloc(sizeof(int32_t) * npix);
    c->q_t = (real*)malloc(sizeof(real) * npix);
    c->p_pos = (vec4*)malloc(sizeof(vec4) * c->P);
    c->p_flux = (vec4*)malloc(sizeof(vec4) * c->P);
    c->p_dir = (vec4*)malloc(sizeof(vec4) * c->P);
    c->p_rng = (vec4*)malloc(sizeof(vec4) * c->P);
    c->p_tri = (int32_t*)malloc(sizeof(int32_t) * c->P);
    c->p_depth = (int32_t*)malloc(sizeof(int32_t) * c->P);
    c->p_t = (real*)malloc(sizeof(real) * c->P);
    c->p_emitted = (uint8_t*)malloc(c->P);
    c->winner = (uint32_t*)malloc(sizeof(uint32_t) * c->hash_num);
    c->count = (uint32_t*)malloc(sizeof(uint32_t) * c->hash_num);
    if (cfg->flags & SPPM_FLAG_PHOTON_GRID) {
        c->g_ofs = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)c->hash_num + 1));
        c->g_ids = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)c->P);
        c->g_cur = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)c->hash_num);
    }
    reset_state(c);
    if (cfg->radius_rule == SPPM_RADIUS_DIAGONAL) {
        const float dx = scene->bbox_max[0] - scene->bbox_min[0];
        const float dy = scene->bbox_max[1] - scene->bbox_min[1];
        const float dz = scene->bbox_max[2] - scene->bbox_min[2];
        c->initial_radius = (real)(cfg->radius_fraction * sqrtf(dx * dx + dy * dy + dz * dz));
    }
    return c;
}

EXPORT void ORACLE_API(reset)(oracle_ctx* c) {
    const real r = c->initial_radius;
    reset_state(c);
    if (c->cfg.radius_rule == SPPM_RADIUS_DIAGONAL) c->initial_radius = r;
}

EXPORT int ORACLE_API(run_frames)(oracle_ctx* c, uint32_t n) {
    for (uint32_t k = 0; k < n && !c->err; k++) run_frame(c);
    return c->err;
}

/* copies one state array in the layout of sppm_read_state (floats; FP64 values are narrowed) */
EXPORT int ORACLE_API(read_state)(oracle_ctx* c, uint32_t kind, void* dst, size_t bytes) {
    const size_t npix = (size_t)c->W * c->H;
    const vec4* v4src = NULL;
    size_t n = 0;
    switch (kind) {
        case SPPM_STATE_HIT_POSITION: v4src = c->q_pos; n = npix; break;
        case SPPM_STATE_HIT_REFLECTANCE: v4src = c->q_refl; n = npix; break;
        case SPPM_STATE_HIT_NORMAL: v4src = c->q_nrm; n = npix; break;
        case SPPM_STATE_EYE_RNG: v4src = c->q_rng; n = npix; break;
        case SPPM_STATE_EMISSION_N: v4src = c->q_emi_n; n = npix; break;
        case SPPM_STATE_FLUX_RADIUS: v4src = c->q_flux_r; n = npix; break;
        case SPPM_STATE_PHOTON_POSITION: v4src = c->p_pos; n = c->P; break;
        case SPPM_STATE_PHOTON_FLUX: v4src = c->p_flux; n = c->P; break;
        case SPPM_STATE_PHOTON_DIRECTION: v4src = c->p_dir; n = c->P; break;
        case SPPM_STATE_PHOTON_RNG: v4src = c->p_rng; n = c->P; break;
        default: break;
    }
    if (v4src) {
        if (bytes != n * 16) return SPPM_ERR_ARG;
        float* o = (float*)dst;
        for (size_t i = 0; i < n; i++) {
            o[i * 4 + 0] = (float)v4src[i].x;
            o[i * 4 + 1] = (float)v4src[i].y;
            o[i * 4 + 2] = (float)v4src[i].z;
            o[i * 4 + 3] = (float)v4src[i].w;
        }
        return 0;
    }
    switch (kind) {
        case SPPM_STATE_HIT_TRIANGLE:
            if (bytes != npix * 4) return SPPM_ERR_ARG;
            memcpy(dst, c->q_tri, bytes);
            return 0;
        case SPPM_STATE_HIT_T: {
            if (bytes != npix * 4) return SPPM_ERR_ARG;
            float* o = (float*)dst;
            for (size_t i = 0; i < npix; i++) o[i] = (float)c->q_t[i];
            return 0;
        }
        case SPPM_STATE_PHOTON_HIT: {
            if (bytes != (size_t)c->P * 8) return SPPM_ERR_ARG;
            int32_t* o = (int32_t*)dst;
            for (size_t i = 0; i < c->P; i++) {
                o[i * 2] = c->p_tri[i];
                o[i * 2 + 1] = c->p_depth[i];
            }
            return 0;
        }
        case SPPM_STATE_SLOT_WINNER:
            if (bytes != (size_t)c->hash_num * 4) return SPPM_ERR_ARG;
            memcpy(dst, c->winner, bytes);
            return 0;
        case SPPM_STATE_SLOT_COUNT:
            if (bytes != (size_t)c->hash_num * 4) return SPPM_ERR_ARG;
            memcpy(dst, c->count, bytes);
            return 0;
        default: return SPPM_ERR_ARG;
    }
}

/* re.fs: kind 0 = linear radiance, 1 = tone-mapped sRGB; rgb is W*H*3 doubles */
EXPORT int ORACLE_API(read_image)(oracle_ctx* c, uint32_t kind, double* rgb, size_t num) {
    const size_t npix = (size_t)c->W * c->H;
    if (num != npix * 3) return SPPM_ERR_ARG;
    const real total = (real)c->num_photons_f32;
    for (size_t p = 0; p < npix; p++) {
        const vec4 fr = c->q_flux_r[p];
        const vec4 qe = c->q_emi_n[p];
        const real R = fr.w;
        const real den = R * R * RC(3.141592) * total;
        real L[3] = {fr.x / den + qe.x, fr.y / den + qe.y, fr.z / den + qe.z};
        for (int k = 0; k < 3; k++) {
            real v = L[k];
            if (kind == SPPM_IMAGE_DISPLAY) {
                v = RC(1.0) - R_EXP(-v * RC(60000.0));
                if (v < RC(0.0031308)) v = RC(12.92) * v;
                else v = (RC(1.0) + RC(0.055)) * R_POW(v, RC(0.416666666667)) - RC(0.055);
            }
            rgb[p * 3 + k] = (double)v;
        }
    }
    return 0;
}

EXPORT void ORACLE_API(frame_info)(oracle_ctx* c, sppm_frame_info* fi) {
    memset(fi, 0, sizeof(*fi));
    fi->frames = c->frame;
    fi->eye_samples = c->eye_samples;
    fi->photons_emitted = c->num_photons;
    fi->num_photons_f32 = c->num_photons_f32;
    fi->initial_radius = (float)c->initial_radius;
    fi->grid_scale = (float)c->grid_scale;
    for (int k = 0; k < 3; k++) {
        fi->bbox_min[k] = (float)c->bbmin[k];
        fi->bbox_max[k] = (float)c->bbmax[k];
    }
    fi->aa_offset[0] = (float)c->aa[0];
    fi->aa_offset[1] = (float)c->aa[1];
    fi->photon_segments = c->photon_segments;
    fi->eye_segments = c->eye_segments;
}

/* stage-level hash build on caller arrays (float4 pos/flux), same contract as sppm_hash_build */
EXPORT void ORACLE_API(hash_build)(const float* pos, const float* flux, uint32_t pw, uint32_t ph, uint32_t hash_slots,
                                   const float bbmin[3], float grid_scale, uint32_t flags, uint32_t* winner,
                                   uint32_t* count) {
    rnd_init_constants();
    const real G = grid_scale;
    const real hs1 = RC(4194304.0) / G;
    const real hn = (real)hash_slots;
    const real pb1 = RC(1.0) / (real)ph;
    for (uint32_t k = 0; k < hash_slots; k++) {
        winner[k] = 0xFFFFFFFFu;
        count[k] = 0;
    }
    for (uint32_t j = 0; j < ph; j++) {
        for (uint32_t i = 0; i < pw; i++) {
            const uint32_t id = j * pw + i;
            if (flux[id * 4] < 0.0f) continue;
            const vec3 cell = v3(R_FLOOR((pos[id * 4] - bbmin[0]) * G), R_FLOOR((pos[id * 4 + 1] - bbmin[1]) * G),
                                 R_FLOOR((pos[id * 4 + 2] - bbmin[2]) * G));
            const uint32_t slot = hash_cell(cell, G, hs1, hn);
            count[slot] += 1;
            const real z = (((real)i + RC(0.5)) / (real)pw) * pb1 + ((real)j + RC(0.5)) / (real)ph;
            if (!(flags & SPPM_FLAG_GL_DEPTH_CLIP) || z < RC(1.0))
                if (id < winner[slot]) winner[slot] = id;
        }
    }
}

/* GPURnd / hash known-answer helpers for tests */
EXPORT void ORACLE_API(gpurnd_sequence)(const float seed[4], uint32_t n, float* out, float* final_state) {
    rnd_init_constants();
    vec4 s = {seed[0], seed[1], seed[2], seed[3]};
    for (uint32_t i = 0; i < n; i++) out[i] = (float)gpu_rnd(&s);
    final_state[0] = (float)s.x;
    final_state[1] = (float)s.y;
    final_state[2] = (float)s.z;
    final_state[3] = (float)s.w;
}

EXPORT uint32_t ORACLE_API(hash_of_cell)(float cx, float cy, float cz, float grid_scale, uint32_t hash_num) {
    rnd_init_constants();
    const real hs1 = RC(4194304.0) / (real)grid_scale;
    return hash_cell(v3(cx, cy, cz), grid_scale, hs1, (real)hash_num);
}

/* ReduceTexture (glslppm.cpp:170-209) with min.fs / max.fs / sum.fs (op 0 / 1 / 2): an R x R
   float4 texture (row 0 first), R a power of two >= 2, folded level by level: the n x n output of a
   level takes texels (i,j), (i+n,j), (i,j+n), (i+n,j+n) of its input, min(min(v0,v1),min(v2,v3)),
   max likewise, or ((v0+v1)+v2)+v3; the result is texel (0,0) after the 1 x 1 level. */
EXPORT int ORACLE_API(reduce_texture)(const float* tex, uint32_t R, uint32_t op, float out[4]) {
    if (R < 2 || (R & (R - 1)) || op > 2) return SPPM_ERR_ARG;
    const uint32_t n1 = R / 2;
    float* w = (float*)malloc(sizeof(float) * 4 * n1 * n1);
    const float* src = tex;
    uint32_t stride = R;
    for (uint32_t n = n1; n >= 1; n /= 2) {
        for (uint32_t j = 0; j < n; j++) {
            for (uint32_t i = 0; i < n; i++) {
                const float* v0 = &src[((size_t)j * stride + i) * 4];
                const float* v1 = &src[((size_t)j * stride + i + n) * 4];
                const float* v2 = &src[((size_t)(j + n) * stride + i) * 4];
                const float* v3 = &src[((size_t)(j + n) * stride + i + n) * 4];
                float r[4];
                for (int c = 0; c < 4; c++) {
                    if (op == 0) r[c] = fminf(fminf(v0[c], v1[c]), fminf(v2[c], v3[c]));
                    else if (op == 1) r[c] = fmaxf(fmaxf(v0[c], v1[c]), fmaxf(v2[c], v3[c]));
                    else r[c] = ((v0[c] + v1[c]) + v2[c]) + v3[c];
                }
                memcpy(&w[((size_t)j * n1 + i) * 4], r, sizeof(r));
            }
        }
        src = w;
        stride = n1;
        if (n == 1) break;
    }
    memcpy(out, w, 4 * sizeof(float));
    free(w);
    return 0;
}

/* raytrace() on single rays against the context's scene: the closest triangle (-1 = none) and
   its t (the initial bound when nothing is hit); photon / cull as in raytrace() */
EXPORT void ORACLE_API(trace)(oracle_ctx* c, const float* org, const float* dir, size_t n, int photon, int cull,
                              int32_t* tri, float* t) {
    for (size_t i = 0; i < n; i++) {
        LastIsect last;
        const vec3 o = v3((real)org[3 * i], (real)org[3 * i + 1], (real)org[3 * i + 2]);
        const vec3 d = v3((real)dir[3 * i], (real)dir[3 * i + 1], (real)dir[3 * i + 2]);
        (void)raytrace(c, o, d, photon, cull, &last);
        tri[i] = last.tri;
        t[i] = (float)last.t;
    }
}

/* the pinned single-precision functions of sppm_fpmath.h evaluated on the host:
   fn 0 sin, 1 cos, 2 pow(x,y), 3 exp, 4 log2, 5 exp2 */
EXPORT void ORACLE_API(fpmath)(int fn, const float* x, const float* y, float* out, size_t n) {
    for (size_t i = 0; i < n; i++) {
        switch (fn) {
            case 0: out[i] = sppm_fsin(x[i]); break;
            case 1: out[i] = sppm_fcos(x[i]); break;
            case 2: out[i] = sppm_fpow(x[i], y[i]); break;
            case 3: out[i] = sppm_fexp(x[i]); break;
            case 4: out[i] = sppm_flog2(x[i]); break;
            default: out[i] = sppm_fexp2(x[i]); break;
        }
    }
}

EXPORT void ORACLE_API(destroy)(oracle_ctx* c) {
    if (!c) return;
    oscene* s = &c->sc;
    free(s->tv);
    free(s->tn);
    free(s->mat);
    free(s->mat_layer);
    free(s->tex);
    free(s->light_tri);
    free(s->light_cdf);
    free(s->nb);
    free(s->ntri);
    free(s->hit_link);
    free(s->miss_link);
    free(c->q_pos);
    free(c->q_refl);
    free(c->q_nrm);
    free(c->q_rng);
    free(c->q_emi_n);
    free(c->q_flux_r);
    free(c->q_tri);
    free(c->q_t);
    free(c->p_pos);
    free(c->p_flux);
    free(c->p_dir);
    free(c->p_rng);
    free(c->p_tri);
    free(c->p_depth);
    free(c->p_t);
    free(c->p_emitted);
    free(c->winner);
    free(c->count);
    free(c->g_ofs);
    free(c->g_ids);
    free(c->g_cur);
    free(c);
}

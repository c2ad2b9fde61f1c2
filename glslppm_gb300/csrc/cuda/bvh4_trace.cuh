// Single-ray traversal of the mixed path's 4-wide quantised BVH (shared by the eye pass of the
// mixed path and the photon kernels of kernels_mixed.cu).
//
// Node4Dev: w[0] = origin xyz, exponent bytes x|y|z|child count; w[1] = the four child links (>= 0
// node, < 0 ~triangle, INT32_MIN empty); w[2] = lower box bytes x,y,z and upper x; w[3] = upper
// y,z.  A child box is origin + byte * 2^(exponent-127) per axis, rounded outward when the tree
// was built; the slab distances are widened by a bound on their rounding, and triangles are
// tested with the exact path's arithmetic (tri_hit_exact), so the closest hit -- triangle, t and
// barycentrics -- is the exact traversal's; where two triangles give the same t, the leaf ranks of
// the exact walk's ordering (DevScene::tri_rank) pick the one it meets first.
#pragma once

#include "device_common.cuh"

namespace sppm_dev {

constexpr int kStack = 196;  // >= 3 * kBvh4MaxDepth + 1 (kBvh4MaxDepth = 64)

struct Hit4 {
    float t;
    int32_t tri;
    float bu, bv, bw;  // (v, w, u) as the plain path stores them
};

__device__ __forceinline__ float node_scale(uint8_t e) { return __uint_as_float((uint32_t)e << 23); }

// direction component used for the slab reciprocals: a zero (or denormal-small) component is
// replaced by +-1e-30 so that the slab of that axis is +-huge instead of NaN (a NaN slab would be
// ignored by fminf/fmaxf and the ray would enter every box the other axes allow)
__device__ __forceinline__ float slab_dir(float d) { return fabsf(d) < 1e-30f ? copysignf(1e-30f, d) : d; }

// byte k of w as an exact float: the byte placed in the low mantissa of 2^23, minus 2^23
__device__ __forceinline__ float byte_f(uint32_t w, uint32_t sel) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, sel)) - 8388608.0f;
}

// ---- conservative slab tests over the quantised boxes ------------------------------------------
// A child plane is P = origin + q * 2^e (q a byte); its distance along the ray is computed as
//     fma(q, A, B -+ E),  A = 2^e * r (exact scaling of r = fl(1/d)),  B = fma(origin, r, n),
//     n = fl(-o * r).
// Against the exact distance (P' - o) / d to the enclosing plane P' = fl(origin + q 2^e) that the
// builder checked, the roundings of r, n, B, B -+ E, the final fma and P' add at most
// 5 u S (1 + O(u)), u = 2^-24, with S = (|origin| + |o| + 255 * 2^e) / |d|
// (each rounding's error is u times a term bounded by S).  E = 16 u S', S' the same sum computed
// from |r|, |n| and |A| (relative error a few u), exceeds that bound, so the near distance is never
// above the exact entry and the far distance never below the exact exit: a box the exact
// arithmetic enters is never culled (Ize, "Robust BVH Ray Traversal", JCGT 2013, applies the same
// argument to the plain slab test).  The near plane of each axis is chosen by the sign of the
// direction once per ray, so a child needs no per-axis min/max.
constexpr float kSlabErr = 9.5367431640625e-07f;  // 16 * 2^-24
// a box entered later than the closest hit so far by less than this relative margin is still
// visited: the exact triangle test's own rounding may put the winner's t just below its box entry
constexpr float kCullMargin = 1.000244140625f;    // 1 + 2^-12

// (|r| and |n| are free operand modifiers; r < 0 selects the upper bound as the near plane)
struct Ray4 {
    float ox, oy, oz, dx, dy, dz;
    float rx, ry, rz, nx, ny, nz;     // r = 1/slab_dir(d), n = -o * r
};

__device__ __forceinline__ void ray4_setup(Ray4& R, float ox, float oy, float oz, float dx, float dy, float dz) {
    R.ox = ox, R.oy = oy, R.oz = oz, R.dx = dx, R.dy = dy, R.dz = dz;
    R.rx = 1.0f / slab_dir(dx), R.ry = 1.0f / slab_dir(dy), R.rz = 1.0f / slab_dir(dz);
    R.nx = -ox * R.rx, R.ny = -oy * R.ry, R.nz = -oz * R.rz;
}

// the node's per-axis slab operands for one ray
struct Slab4 {
    float Ax, Ay, Az;        // 2^e * r
    float Nx, Ny, Nz;        // B - E (near planes)
    float Fx, Fy, Fz;        // B + E (far planes)
    uint32_t nwx, nwy, nwz;  // words holding the near-plane bytes of the four children
    uint32_t fwx, fwy, fwz;  // ... and the far-plane bytes
};

__device__ __forceinline__ float slab_err(float origin, float r, float n, float A) {
    return kSlabErr * fmaf(255.0f, fabsf(A), fmaf(fabsf(origin), fabsf(r), fabsf(n)));
}

__device__ __forceinline__ void slab4_setup(Slab4& S, const Ray4& R, const float4& w0, const float4& w2,
                                            const float4& w3) {
    const uint32_t eb = __float_as_uint(w0.w);
    S.Ax = node_scale(eb & 0xFF) * R.rx;
    S.Ay = node_scale((eb >> 8) & 0xFF) * R.ry;
    S.Az = node_scale((eb >> 16) & 0xFF) * R.rz;
    const float Bx = fmaf(w0.x, R.rx, R.nx), By = fmaf(w0.y, R.ry, R.ny), Bz = fmaf(w0.z, R.rz, R.nz);
    const float Ex = slab_err(w0.x, R.rx, R.nx, S.Ax);
    const float Ey = slab_err(w0.y, R.ry, R.ny, S.Ay);
    const float Ez = slab_err(w0.z, R.rz, R.nz, S.Az);
    S.Nx = Bx - Ex, S.Ny = By - Ey, S.Nz = Bz - Ez;
    S.Fx = Bx + Ex, S.Fy = By + Ey, S.Fz = Bz + Ez;
    // lower bytes: x w2.x, y w2.y, z w2.z; upper bytes: x w2.w, y w3.x, z w3.y
    const uint32_t lx = __float_as_uint(w2.x), ly = __float_as_uint(w2.y), lz = __float_as_uint(w2.z);
    const uint32_t hx = __float_as_uint(w2.w), hy = __float_as_uint(w3.x), hz = __float_as_uint(w3.y);
    const bool negx = R.rx < 0.0f, negy = R.ry < 0.0f, negz = R.rz < 0.0f;
    S.nwx = negx ? hx : lx, S.fwx = negx ? lx : hx;
    S.nwy = negy ? hy : ly, S.fwy = negy ? ly : hy;
    S.nwz = negz ? hz : lz, S.fwz = negz ? lz : hz;
}

// conservative entry distance of child K (clamped at 0) and whether the ray may hit its box before
// tcull (the closest hit so far times kCullMargin)
template <int K>
__device__ __forceinline__ void child_box(const Slab4& S, float tcull, float& tn, bool& hit) {
    constexpr uint32_t sel = 0x7650u | (uint32_t)K;  // byte K of the word into byte 0, 0x4B into byte 3
    const float nx = fmaf(byte_f(S.nwx, sel), S.Ax, S.Nx);
    const float ny = fmaf(byte_f(S.nwy, sel), S.Ay, S.Ny);
    const float nz = fmaf(byte_f(S.nwz, sel), S.Az, S.Nz);
    const float fx = fmaf(byte_f(S.fwx, sel), S.Ax, S.Fx);
    const float fy = fmaf(byte_f(S.fwy, sel), S.Ay, S.Fy);
    const float fz = fmaf(byte_f(S.fwz, sel), S.Az, S.Fz);
    const float t0 = fmaxf(fmax3(nx, ny, nz), 0.0f);
    const float t1 = fmin3(fx, fy, fz);
    tn = t0;
    hit = t0 <= t1 && t0 <= tcull;
}

__device__ __forceinline__ void cswap(float& ta, int32_t& ca, float& tb, int32_t& cb) {
    if (tb < ta) {
        const float t = ta;
        ta = tb;
        tb = t;
        const int32_t c = ca;
        ca = cb;
        cb = c;
    }
}

// closest hit through the 4-wide BVH; PHOTON rays skip emitters, eye rays of the first bounce
// cull back faces (eyeraytrace.fs:130)
// rank: the leaf positions of the ordering the exact walk would take for this ray (tri_rank of
// its cube face) or null; at an equal t the triangle the exact walk meets first wins, as there
template <bool PHOTON>
__device__ __forceinline__ Hit4 trace4(const Node4Dev* __restrict__ nodes, const float4* __restrict__ tri_isect, f3 org,
                                       f3 dir, bool cull, float tmax0, uint32_t& err,
                                       const int32_t* __restrict__ rank = nullptr) {
    Hit4 h;
    h.t = tmax0;
    h.tri = -1;
    h.bu = h.bv = h.bw = 0.0f;
    Ray4 R;
    ray4_setup(R, org.x, org.y, org.z, dir.x, dir.y, dir.z);
    int32_t stack_node[kStack];
    float stack_t[kStack];
    int sp = 0;
    int32_t cur = 0;
    uint32_t visits = 0;
    for (;;) {
        if (++visits > 4u * (1u << 20)) {  // bounded: no tree here has this many nodes
            err |= kErrWatchdogTraverse;
            break;
        }
        const float4* np = reinterpret_cast<const float4*>(nodes + cur);
        float4 w0, w1, w2, w3;
        ldg32(np, w0, w1);
        ldg32(np + 2, w2, w3);
        const int cnt = (int)(__float_as_uint(w0.w) >> 24);
        int32_t ch[4] = {__float_as_int(w1.x), __float_as_int(w1.y), __float_as_int(w1.z), __float_as_int(w1.w)};
        // conservative slab test of the (up to) four children
        float tnear[4];
        bool hit[4];
        Slab4 S;
        slab4_setup(S, R, w0, w2, w3);
        const float tcull = h.t * kCullMargin;
        child_box<0>(S, tcull, tnear[0], hit[0]);
        child_box<1>(S, tcull, tnear[1], hit[1]);
        child_box<2>(S, tcull, tnear[2], hit[2]);
        child_box<3>(S, tcull, tnear[3], hit[3]);
        // leaf children: their triangles in child order (a closer hit shrinks the search), one copy
        // of the test in a loop over the leaves
        uint32_t leaves = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            hit[k] = hit[k] && k < cnt;
            if (!hit[k] || ch[k] >= 0) continue;
            hit[k] = false;
            if (!(PHOTON && (~ch[k] & kEmitterBit))) leaves |= 1u << k;
        }
        while (leaves) {
            const int k = __ffs(leaves) - 1;
            leaves &= leaves - 1;
            const int32_t ck = k == 0 ? ch[0] : (k == 1 ? ch[1] : (k == 2 ? ch[2] : ch[3]));
            const int32_t tri = ~ck & kTriMask;
            const float4 a = __ldg(&tri_isect[(size_t)tri * 3 + 0]);
            const float4 b = __ldg(&tri_isect[(size_t)tri * 3 + 1]);
            const float4 c = __ldg(&tri_isect[(size_t)tri * 3 + 2]);
            float tt, u, v, w;
            if (tri_hit_exact(a, b, c, org, dir, !PHOTON && cull, tt, u, v, w) &&
                (tt < h.t || (rank && tt == h.t && h.tri >= 0 && __ldg(&rank[tri]) < __ldg(&rank[h.tri])))) {
                h.t = tt;
                h.tri = tri;
                h.bu = v;
                h.bv = w;
                h.bw = u;
            }
        }
        // internal children hit before the closest hit so far, sorted near to far: the nearest
        // is next, the others go on the stack farthest first
        const float inf = __int_as_float(0x7f800000);
        const float tcull2 = h.t * kCullMargin;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (!(hit[k] && tnear[k] <= tcull2)) tnear[k] = inf;
        cswap(tnear[0], ch[0], tnear[1], ch[1]);
        cswap(tnear[2], ch[2], tnear[3], ch[3]);
        cswap(tnear[0], ch[0], tnear[2], ch[2]);
        cswap(tnear[1], ch[1], tnear[3], ch[3]);
        cswap(tnear[1], ch[1], tnear[2], ch[2]);
        if (tnear[0] < inf) {
            const int pushes = (tnear[1] < inf) + (tnear[2] < inf) + (tnear[3] < inf);
            if (sp + pushes > kStack) {
                err |= kErrWatchdogTraverse;
                break;
            }
            if (tnear[3] < inf) stack_node[sp] = ch[3], stack_t[sp++] = tnear[3];
            if (tnear[2] < inf) stack_node[sp] = ch[2], stack_t[sp++] = tnear[2];
            if (tnear[1] < inf) stack_node[sp] = ch[1], stack_t[sp++] = tnear[1];
            cur = ch[0];
            continue;
        }
        bool found = false;
        while (sp > 0) {
            sp--;
            if (stack_t[sp] <= h.t * kCullMargin) {
                cur = stack_node[sp];
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    return h;
}


}  // namespace sppm_dev

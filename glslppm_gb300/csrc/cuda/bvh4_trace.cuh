// Single-ray traversal of the mixed path's 4-wide quantised BVH (shared by the eye pass of the
// mixed path and the photon kernels of kernels_mixed.cu).
//
// Node4Dev: w[0] = origin xyz, exponent bytes x|y|z|child count; w[1] = the four child links (>= 0
// node, < 0 ~triangle, INT32_MIN empty); w[2] = lower box bytes x,y,z and upper x; w[3] = upper
// y,z.  A child box is origin + byte * 2^(exponent-127) per axis, rounded outward when the tree
// was built, so the slab tests are conservative.
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

// slab distances of child K's box: plane = origin + byte * 2^e, so its distance along the ray is
// byte * (2^e / d) + (origin - o) / d = fmaf(byte, A, B) with the per-node A = 2^e * (1/d) (exact:
// a power-of-two scale) and B = fmaf(origin, 1/d, -o/d)
template <int K>
__device__ __forceinline__ void child_box(const float4& w2, const float4& w3, float Ax, float Ay, float Az, float Bx,
                                          float By, float Bz, float tbest, float& tn, bool& hit) {
    constexpr uint32_t sel = 0x7650u | (uint32_t)K;  // byte K of the word into byte 0, 0x4B into byte 3
    const float ax = fmaf(byte_f(__float_as_uint(w2.x), sel), Ax, Bx);
    const float ay = fmaf(byte_f(__float_as_uint(w2.y), sel), Ay, By);
    const float az = fmaf(byte_f(__float_as_uint(w2.z), sel), Az, Bz);
    const float bx = fmaf(byte_f(__float_as_uint(w2.w), sel), Ax, Bx);
    const float by = fmaf(byte_f(__float_as_uint(w3.x), sel), Ay, By);
    const float bz = fmaf(byte_f(__float_as_uint(w3.y), sel), Az, Bz);
    const float t0 = fmaxf(fmax3(fminf(ax, bx), fminf(ay, by), fminf(az, bz)), 0.0f);
    // the far bound widened by a few ulps so that rounding never rejects a grazing hit
    const float t1 = fmin3(fmaxf(ax, bx), fmaxf(ay, by), fmaxf(az, bz)) * 1.00000036f;
    tn = t0;
    hit = t0 <= t1 && t0 <= tbest;
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
template <bool PHOTON>
__device__ __forceinline__ Hit4 trace4(const Node4Dev* __restrict__ nodes, const float4* __restrict__ tri_isect, f3 org,
                                       f3 dir, bool cull, float tmax0, uint32_t& err) {
    Hit4 h;
    h.t = tmax0;
    h.tri = -1;
    h.bu = h.bv = h.bw = 0.0f;
    const float rx = 1.0f / slab_dir(dir.x), ry = 1.0f / slab_dir(dir.y), rz = 1.0f / slab_dir(dir.z);
    const float nx = -org.x * rx, ny = -org.y * ry, nz = -org.z * rz;
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
        const uint32_t eb = __float_as_uint(w0.w);
        const float sx = node_scale(eb & 0xFF), sy = node_scale((eb >> 8) & 0xFF), sz = node_scale((eb >> 16) & 0xFF);
        const int cnt = (int)(eb >> 24);
        int32_t ch[4] = {__float_as_int(w1.x), __float_as_int(w1.y), __float_as_int(w1.z), __float_as_int(w1.w)};
        // slab test of the (up to) four children
        float tnear[4];
        bool hit[4];
        const float Ax = sx * rx, Ay = sy * ry, Az = sz * rz;
        const float Bx = fmaf(w0.x, rx, nx), By = fmaf(w0.y, ry, ny), Bz = fmaf(w0.z, rz, nz);
        child_box<0>(w2, w3, Ax, Ay, Az, Bx, By, Bz, h.t, tnear[0], hit[0]);
        child_box<1>(w2, w3, Ax, Ay, Az, Bx, By, Bz, h.t, tnear[1], hit[1]);
        child_box<2>(w2, w3, Ax, Ay, Az, Bx, By, Bz, h.t, tnear[2], hit[2]);
        child_box<3>(w2, w3, Ax, Ay, Az, Bx, By, Bz, h.t, tnear[3], hit[3]);
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
            const f3 e0 = mk(a.w, b.x, b.y), e1 = mk(b.z, b.w, c.x);
            const float pvx = dir.y * e1.z - dir.z * e1.y, pvy = dir.z * e1.x - dir.x * e1.z,
                        pvz = dir.x * e1.y - dir.y * e1.x;
            const float det = e0.x * pvx + e0.y * pvy + e0.z * pvz;
            if (!PHOTON && cull && !(det > 1e-10f)) continue;
            const float inv = 1.0f / det;
            const float tvx = org.x - a.x, tvy = org.y - a.y, tvz = org.z - a.z;
            const float u = (tvx * pvx + tvy * pvy + tvz * pvz) * inv;
            if (!(u >= 0.0f && u <= 1.0f)) continue;
            const float qx = tvy * e0.z - tvz * e0.y, qy = tvz * e0.x - tvx * e0.z, qz = tvx * e0.y - tvy * e0.x;
            const float v = (dir.x * qx + dir.y * qy + dir.z * qz) * inv;
            const float t = (e1.x * qx + e1.y * qy + e1.z * qz) * inv;
            const float w = 1.0f - u - v;
            if (v >= 0.0f && w >= 0.0f && t >= 0.0f && t < h.t) {
                h.t = t;
                h.tri = tri;
                h.bu = v;
                h.bv = w;
                h.bw = u;
            }
        }
        // internal children hit before the closest hit so far, sorted near to far: the nearest
        // is next, the others go on the stack farthest first
        const float inf = __int_as_float(0x7f800000);
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (!(hit[k] && tnear[k] <= h.t)) tnear[k] = inf;
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
            if (stack_t[sp] <= h.t) {
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

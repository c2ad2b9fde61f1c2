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
        const int32_t ch[4] = {__float_as_int(w1.x), __float_as_int(w1.y), __float_as_int(w1.z), __float_as_int(w1.w)};
        const uint32_t qlx = __float_as_uint(w2.x), qly = __float_as_uint(w2.y), qlz = __float_as_uint(w2.z);
        const uint32_t qhx = __float_as_uint(w2.w), qhy = __float_as_uint(w3.x), qhz = __float_as_uint(w3.y);
        // slab test of the (up to) four children
        float tnear[4];
        bool hit[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float lx = fmaf((float)((qlx >> (8 * k)) & 0xFF), sx, w0.x);
            const float ly = fmaf((float)((qly >> (8 * k)) & 0xFF), sy, w0.y);
            const float lz = fmaf((float)((qlz >> (8 * k)) & 0xFF), sz, w0.z);
            const float hx = fmaf((float)((qhx >> (8 * k)) & 0xFF), sx, w0.x);
            const float hy = fmaf((float)((qhy >> (8 * k)) & 0xFF), sy, w0.y);
            const float hz = fmaf((float)((qhz >> (8 * k)) & 0xFF), sz, w0.z);
            const float ax = fmaf(lx, rx, nx), bx = fmaf(hx, rx, nx);
            const float ay = fmaf(ly, ry, ny), by = fmaf(hy, ry, ny);
            const float az = fmaf(lz, rz, nz), bz = fmaf(hz, rz, nz);
            const float t0 = fmaxf(fmax3(fminf(ax, bx), fminf(ay, by), fminf(az, bz)), 0.0f);
            // widen the far bound by a few ulps so that rounding never rejects a grazing hit
            const float t1 = fmin3(fmaxf(ax, bx), fmaxf(ay, by), fmaxf(az, bz)) * 1.00000036f;
            tnear[k] = t0;
            hit[k] = k < cnt && t0 <= t1 && t0 <= h.t;
        }
        // leaf children: test their triangle now (a closer hit shrinks the search)
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (!hit[k] || ch[k] >= 0) continue;
            hit[k] = false;
            const int32_t code = ~ch[k];
            if (PHOTON && (code & kEmitterBit)) continue;
            const int32_t tri = code & kTriMask;
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
        // internal children: nearest next, the others on the stack (farthest first)
        int32_t order[4];
        float ot[4];
        int n = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (hit[k] && tnear[k] <= h.t) {
                int j = n++;
                while (j > 0 && ot[j - 1] < tnear[k]) {  // descending distance
                    ot[j] = ot[j - 1];
                    order[j] = order[j - 1];
                    j--;
                }
                ot[j] = tnear[k];
                order[j] = ch[k];
            }
        }
        if (n > 0) {
            if (sp + n - 1 > kStack) {
                err |= kErrWatchdogTraverse;
                break;
            }
            for (int j = 0; j < n - 1; j++) {
                stack_node[sp] = order[j];
                stack_t[sp] = ot[j];
                sp++;
            }
            cur = order[n - 1];
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

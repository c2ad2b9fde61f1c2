// ReduceTexture (glslppm.cpp:170-209) as a stage-level entry point.
//
// The reference reduces an R x R RGBA32F texture to one texel by drawing quads of R/2, R/4, ... 1
// pixels into a ping-pong texture; each output texel applies min.fs / max.fs / sum.fs to the four
// texels (i,j), (i+n,j), (i,j+n), (i+n,j+n) of the previous level, and the host reads texel (0,0).
// One kernel launch per level restates it; the levels after the first run in place on a
// (R/2) x (R/2) float4 scratch buffer (a thread reads its own output texel and three texels outside
// the level's output square, so no thread reads what another writes).  The sums are evaluated as
// ((v0 + v1) + v2) + v3 with non-fused adds, so all three results are bit-identical to the
// reference's fold.
#include <cstdint>
#include <mutex>

#include <cuda.h>  // driver types only (CUcontext, CUresult); nothing is linked
#include <cuda_runtime.h>

#include "../host/scene_internal.h"
#include "device_common.cuh"

namespace sppm_dev {

__global__ void k_reduce_level(const float4* src, uint32_t src_stride, float4* dst, uint32_t dst_stride,
                               uint32_t n, uint32_t op) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const uint32_t i = t % n, j = t / n;
    const float4 v0 = src[(size_t)j * src_stride + i];
    const float4 v1 = src[(size_t)j * src_stride + i + n];
    const float4 v2 = src[(size_t)(j + n) * src_stride + i];
    const float4 v3 = src[(size_t)(j + n) * src_stride + i + n];
    float4 r;
    if (op == SPPM_REDUCE_MIN) {
        r = make_float4(fminf(fminf(v0.x, v1.x), fminf(v2.x, v3.x)), fminf(fminf(v0.y, v1.y), fminf(v2.y, v3.y)),
                        fminf(fminf(v0.z, v1.z), fminf(v2.z, v3.z)), fminf(fminf(v0.w, v1.w), fminf(v2.w, v3.w)));
    } else if (op == SPPM_REDUCE_MAX) {
        r = make_float4(fmaxf(fmaxf(v0.x, v1.x), fmaxf(v2.x, v3.x)), fmaxf(fmaxf(v0.y, v1.y), fmaxf(v2.y, v3.y)),
                        fmaxf(fmaxf(v0.z, v1.z), fmaxf(v2.z, v3.z)), fmaxf(fmaxf(v0.w, v1.w), fmaxf(v2.w, v3.w)));
    } else {
        r = make_float4(__fadd_rn(__fadd_rn(__fadd_rn(v0.x, v1.x), v2.x), v3.x),
                        __fadd_rn(__fadd_rn(__fadd_rn(v0.y, v1.y), v2.y), v3.y),
                        __fadd_rn(__fadd_rn(__fadd_rn(v0.z, v1.z), v2.z), v3.z),
                        __fadd_rn(__fadd_rn(__fadd_rn(v0.w, v1.w), v2.w), v3.w));
    }
    dst[(size_t)j * dst_stride + i] = r;
}

// all levels of one reduction; the result is scratch[0] when the last launch completes
void launch_reduce_texture(const float4* tex, uint32_t resolution, uint32_t op, float4* scratch, cudaStream_t s) {
    const uint32_t n1 = resolution / 2;
    const float4* src = tex;
    uint32_t stride = resolution;
    for (uint32_t n = n1; n >= 1; n /= 2) {
        const uint32_t items = n * n;
        k_reduce_level<<<(items + 255) / 256, 256, 0, s>>>(src, stride, scratch, n1, n, op);
        src = scratch;
        stride = n1;
        if (n == 1) break;
    }
}

}  // namespace sppm_dev

using sppm::fail;

// ---- variant without device allocation ---------------------------------------------------------
// Its scratch is this file-scope device array: 512 x 512 float4 = 4 MiB, held by every GPU that
// loads the library until the process exits.  Host code must not pass `g_reduce_scratch` itself to a
// kernel (on the host it names a host-side shadow, not device memory): the device address is looked
// up with cudaGetSymbolAddress once per device and context, with that device current, and cached.
static __device__ __align__(256) float4 g_reduce_scratch[(SPPM_REDUCE_NOALLOC_MAX_RESOLUTION / 2) *
                                                         (SPPM_REDUCE_NOALLOC_MAX_RESOLUTION / 2)];

namespace {
// The device address of g_reduce_scratch belongs to the CUDA context that loaded the library's
// device code: a device reset (cudaDeviceReset) destroys that context and the next runtime call
// creates a new one, in which the array may sit elsewhere.  The cache is therefore keyed on the
// context's unique id (cuCtxGetId, never reused within a process), read through driver entry
// points that the runtime hands out, so the library needs no link against the driver library.
typedef CUresult (*PFN_ctx_get_current)(CUcontext*);
typedef CUresult (*PFN_ctx_get_id)(CUcontext, unsigned long long*);

struct ScratchEntry {
    unsigned long long ctx_id;
    float4* ptr;
};
std::mutex g_scratch_mutex;
ScratchEntry g_scratch_cache[64];  // per device ordinal: the context it was looked up in, address
PFN_ctx_get_current g_ctx_get_current = nullptr;
PFN_ctx_get_id g_ctx_get_id = nullptr;

// id of the current context, 0 when none is current (after a reset, before the next runtime call)
int current_context_id(unsigned long long* id) {
    *id = 0;
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return fail(SPPM_ERR_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId unavailable: %s",
                        cudaGetErrorString(e));
        g_ctx_get_current = reinterpret_cast<PFN_ctx_get_current>(f1);
        g_ctx_get_id = reinterpret_cast<PFN_ctx_get_id>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return fail(SPPM_ERR_CUDA, "cuCtxGetCurrent failed");
    if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return fail(SPPM_ERR_CUDA, "cuCtxGetId failed");
    return SPPM_OK;
}

// Set-up of the entry point: on the first call in a device's current context (and again after a
// device reset replaced that context), the array's device address is looked up with that device
// current and cached; later calls in the same context reuse it.
int scratch_address(float4** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SPPM_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(SPPM_ERR_ARG, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    unsigned long long id = 0;
    int st = current_context_id(&id);
    if (st) return st;
    ScratchEntry& c = g_scratch_cache[dev];
    if (id == 0 || !c.ptr || c.ctx_id != id) {
        // also makes the device's primary context current when none is
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_reduce_scratch);
        if (e != cudaSuccess || !p)
            return fail(SPPM_ERR_CUDA, "cudaGetSymbolAddress(g_reduce_scratch) failed: %s", cudaGetErrorString(e));
        if (id == 0 && (st = current_context_id(&id)) != SPPM_OK) return st;
        c.ptr = static_cast<float4*>(p);
        c.ctx_id = id;
    }
    *out = c.ptr;
    return SPPM_OK;
}
}  // namespace

extern "C" int sppm_reduce_texture_noalloc(const float* d_texture, uint32_t resolution, uint32_t op, float out[4],
                                           void* stream) {
    if (!d_texture || !out) return fail(SPPM_ERR_ARG, "sppm_reduce_texture_noalloc: null argument");
    if (resolution < 2 || (resolution & (resolution - 1)))
        return fail(SPPM_ERR_ARG, "sppm_reduce_texture_noalloc: resolution %u must be a power of two >= 2", resolution);
    if (resolution > SPPM_REDUCE_NOALLOC_MAX_RESOLUTION)
        return fail(SPPM_ERR_ARG,
                    "sppm_reduce_texture_noalloc: resolution %u exceeds the maximum %u of its fixed scratch "
                    "(use sppm_reduce_texture)", resolution, (unsigned)SPPM_REDUCE_NOALLOC_MAX_RESOLUTION);
    if (op > SPPM_REDUCE_SUM) return fail(SPPM_ERR_ARG, "sppm_reduce_texture_noalloc: unknown op %u", op);
    if (reinterpret_cast<uintptr_t>(d_texture) & 15) return fail(SPPM_ERR_ARG, "texture must be 16-byte aligned");
    float4* scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // no clearing needed: every level writes each scratch texel it later reads
    sppm_dev::launch_reduce_texture(reinterpret_cast<const float4*>(d_texture), resolution, op, scratch, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, scratch, sizeof(float4), cudaMemcpyDeviceToHost, s);
    const cudaError_t e2 = cudaStreamSynchronize(s);
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(SPPM_ERR_CUDA, "sppm_reduce_texture_noalloc failed: %s",
                    cudaGetErrorString(e != cudaSuccess ? e : e2));
    return SPPM_OK;
}

extern "C" int sppm_reduce_texture(const float* d_texture, uint32_t resolution, uint32_t op, float out[4],
                                   void* stream) {
    if (!d_texture || !out) return fail(SPPM_ERR_ARG, "sppm_reduce_texture: null argument");
    if (resolution < 2 || (resolution & (resolution - 1)) || resolution > 16384)
        return fail(SPPM_ERR_ARG, "sppm_reduce_texture: resolution %u must be a power of two in [2, 16384]", resolution);
    if (op > SPPM_REDUCE_SUM) return fail(SPPM_ERR_ARG, "sppm_reduce_texture: unknown op %u", op);
    if (reinterpret_cast<uintptr_t>(d_texture) & 15) return fail(SPPM_ERR_ARG, "texture must be 16-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n1 = resolution / 2;
    float4* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, n1 * n1 * sizeof(float4), s);
    if (e != cudaSuccess) return fail(SPPM_ERR_OOM, "sppm_reduce_texture: scratch allocation failed: %s", cudaGetErrorString(e));
    sppm_dev::launch_reduce_texture(reinterpret_cast<const float4*>(d_texture), resolution, op, scratch, s);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, scratch, sizeof(float4), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(scratch, s);
    const cudaError_t e2 = cudaStreamSynchronize(s);
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(SPPM_ERR_CUDA, "sppm_reduce_texture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    return SPPM_OK;
}

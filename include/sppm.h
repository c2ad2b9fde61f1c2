/*
 * sppm.h -- C ABI of the GB300 (sm_103a) stochastic progressive photon mapping path.
 *
 * This library replaces the OpenGL shader path of glslppm (T. Hachisuka, Tokyo Demo Fest 2015,
 * modified by tigrazone).  In the reference, the host class CGPURT (gpurt.h:29-67) packs the
 * scene built by TMesh (mesh.cpp) and TBVH (bvh.cpp) into RGBA32F textures, and m_display()
 * (glslppm.cpp:214-536) drives one SPPM frame as a chain of fragment/vertex-shader draws:
 *
 *   eyeraytrace.fs -> ReduceTexture(max/min) -> photontrace.fs -> ReduceTexture(sum)
 *   -> hash.fs -> scatter.vs/.fs (depth test) -> correction.vs/.fs (blend) -> progressive.fs
 *   -> re.fs
 *
 * Every entry point below takes plain pointers and sizes; no GL, torch or C++ type crosses the
 * boundary.  All entry points return an sppm_status (0 = success); the message of the last
 * failure on the calling thread is available from sppm_last_error().  No entry point calls
 * exit() or lets a C++ exception escape.
 *
 * Threading: a context is used by one host thread at a time.  Work is queued on the context's
 * CUDA stream; sppm_synchronize() waits for it and reports device-side errors (for example a
 * BVH traversal that exceeded its step bound because the scene's links are corrupt).
 */
#ifndef SPPM_H
#define SPPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPPM_ABI_VERSION 1

/* ---- status codes ----------------------------------------------------------------------------- */
typedef enum sppm_status {
    SPPM_OK = 0,
    SPPM_ERR_ARG = 1,         /* invalid argument (null pointer, size mismatch, bad enum)          */
    SPPM_ERR_OOM = 2,         /* device or host allocation failed, or admission limit exceeded     */
    SPPM_ERR_CUDA = 3,        /* a CUDA runtime call failed                                         */
    SPPM_ERR_WATCHDOG = 4,    /* a bounded device loop gave up (corrupt BVH links, bad light table) */
    SPPM_ERR_STATE = 5,       /* call out of order (e.g. run before a scene is uploaded)            */
    SPPM_ERR_IO = 6,          /* file could not be opened or parsed                                 */
    SPPM_ERR_UNSUPPORTED = 7, /* feature not available in this build                                */
    SPPM_ERR_NO_DEVICE = 8    /* no CUDA device                                                     */
} sppm_status;

/* ---- configuration ---------------------------------------------------------------------------- */
typedef enum sppm_precision {
    /* Plain FP32: every operation of the reference shaders in IEEE single precision, in the order
       the shaders write it, transcendentals from sppm_fpmath.h.  Bit-identical to the CPU
       restatement of the shaders. */
    SPPM_PRECISION_FP32 = 0,
    /* Mixed: 4-wide traversal over outward-rounded quantised child boxes (FMA slab tests widened
       by their rounding bound, the exact triangle test, ties at equal t in the exact walk's order:
       the plain walk's hits, or a closer triangle where the plain walk's rounded box test skips
       one), photon flux and direction stored in FP16, flux gathered in FP32, per-pixel N, R^2 and
       tau as double-float pairs (read as doubles). */
    SPPM_PRECISION_MIXED = 1
} sppm_precision;

typedef enum sppm_radius_rule {
    /* InitialRadius = (mean extent of the hit-point bounding box) / width * footprint,
       recomputed after every eye pass (glslppm.cpp:294-311). */
    SPPM_RADIUS_FOOTPRINT = 0,
    /* InitialRadius = radius_fraction * |scene bbox diagonal| (a fixed radius). */
    SPPM_RADIUS_DIAGONAL = 1
} sppm_radius_rule;

typedef enum sppm_seed_mode {
    /* Xorshift128 fills the eye, then the photon random-state tables at start, row-major, and
       draws the anti-aliasing offset of each eye pass (glslppm.cpp:77-140, 276-278).  With
       seed = 0 the stream starts from the reference's constants. */
    SPPM_SEED_XORSHIFT = 0,
    /* Per-pixel and per-photon state from an integer hash of (seed, index): no host fill. */
    SPPM_SEED_HASH = 1
} sppm_seed_mode;

/* Flags */
#define SPPM_FLAG_FUSED_PHOTON 0x2u  /* one photon kernel per pass instead of the wavefront
                                        generate -> trace -> store (same results) */
#define SPPM_FLAG_GL_DEPTH_CLIP 0x1u /* scatter.vs: photons whose depth z >= 1 (last row, i >= w/2)
                                        are counted but never become a slot's stored photon */
#define SPPM_FLAG_EAGER_LAUNCH 0x8u  /* launch each frame's kernels one by one instead of replaying the
                                        frame's CUDA graph (same results) */
#define SPPM_FLAG_UNBINNED_RAYS 0x4u /* wavefront pass: trace the photon rays in queue order instead
                                        of binned by direction class and origin cell (same results) */
#define SPPM_FLAG_FP64_STATISTICS 0x10u /* mixed precision only: keep N, R^2 and tau in IEEE double and
                                           update them in FP64 arithmetic instead of double-float
                                           pairs (same memory; the GPU's FP64 rate makes the gather
                                           slower) */
#define SPPM_FLAG_PHOTON_GRID 0x20u /* mixed precision only: the counting-sort photon grid.  After each
                                       photon pass every stored photon is sorted by hash slot (the
                                       slots' photon counts, an exclusive scan, a scatter of 16-byte
                                       records: position in 21-bit grid fixed point, FP16 flux, 8-bit
                                       octahedral direction), and the gather sums EVERY photon of the
                                       2x2x2 cells within the radius instead of the slot's winner times
                                       the slot's count.  The cells, the hash and the radius update are
                                       the reference's; the per-pass estimate has the same expectation
                                       and a far smaller variance (the image differs from the plain
                                       path's, converging to the same limit).  Flux sums are exact
                                       (integer), so results do not depend on the order of the sort. */

typedef struct sppm_config {
    uint32_t width, height;               /* image (ImageResolution x ImageResolution in the ref)  */
    uint32_t photon_width, photon_height; /* photon slots, P = w*h per pass (PhotonBufferSize^2)  */
    uint32_t hash_slots;                  /* HashNum; 0 means P (HashResolution^2 in the ref)      */
    uint32_t max_path_length;             /* MaxNumberOfBounces = 10 (glslppm.cpp:36)              */
    uint32_t eye_pass_interval;           /* eye pass every N frames; 10 in the ref (:238)         */
    float alpha;                          /* 0.7 (glslppm.cpp:488)                                 */
    float initial_footprint;              /* 2.5 (glslppm.cpp:40)                                  */
    uint32_t radius_rule;                 /* sppm_radius_rule                                      */
    float radius_fraction;                /* for SPPM_RADIUS_DIAGONAL                              */
    uint32_t precision;                   /* sppm_precision                                        */
    uint32_t seed_mode;                   /* sppm_seed_mode                                        */
    uint32_t seed;                        /* 0 = the reference's xorshift constants                */
    uint32_t flags;                       /* SPPM_FLAG_*                                           */
    float focal_length;                   /* 13 (glslppm.cpp:31)                                   */
    float aperture;                       /* 0  (glslppm.cpp:32)                                   */
} sppm_config;

/* Fills *cfg with the reference's constants for a square image of side `resolution`. */
void sppm_config_defaults(sppm_config* cfg, uint32_t resolution);

/* ---- scene -------------------------------------------------------------------------------------
 * Mirrors TMesh (mesh.h:49-67) and TBVH (bvh.h:24-33) after TMesh::LoadOBJ and TBVH::Build.
 * Material fields are the ones CGPURT::CreateTextures packs (gpurt.cpp:109-132).               */
typedef struct sppm_material {
    float color[3];   /* TMaterial::color (diffuse already x0.9 for brdf 0/3, mesh.cpp:591-594) */
    float eta;        /* TMaterial::eta                                                         */
    int32_t brdf;     /* -1 light, 0 matte, 1 mirror, 2 glass, 3 plastic, 4/5/6 glossy, 7 sss   */
    float glossiness; /* 1/((2/(1-specularity))^2.71828 + 1), the packed g (gpurt.cpp:126)      */
} sppm_material;

typedef struct sppm_scene {
    uint32_t num_triangles;
    const float* positions;       /* [n][3 vertices][xyz]  TTriangle::positions                  */
    const float* normals;         /* [n][3][xyz]           TTriangle::normals                    */
    const float* texcoords;       /* [n][3][uv] or NULL    TTriangle::texcoords (1e30 = none)    */
    const int32_t* material_ids;  /* [n]                   TTriangle::idMaterial                 */
    uint32_t num_materials;
    const sppm_material* materials;
    uint32_t num_lights;
    const int32_t* light_triangles; /* TMesh::lightsIndices                                      */
    const float* light_cdf;         /* TMesh::lightsCDF (normalised, ascending)                  */
    float light_area;               /* TMesh::lightsArea; 0 means image-based light (IBL)        */
    float bbox_min[3], bbox_max[3]; /* TMesh::bbox                                               */
    /* TBVH after Build(): 2n-1 nodes; node arrays of the canonical ordering (face 0) ... */
    uint32_t num_nodes;
    const float* node_bounds;      /* [num_nodes][6] = min xyz, max xyz of nodes[0][i].bbox      */
    const int32_t* node_triangle;  /* [num_nodes] nodes[0][i].idTriangle for leaves, -1 else     */
    /* ... and for each of the 6 orderings o (+x,-x,+y,-y,+z,-z), the traversal sequence:      */
    const int32_t* order_base;     /* [6][num_nodes] nodes[o][i].idBase (canonical id)           */
    const int32_t* order_miss;     /* [6][num_nodes] nodes[o][i].idMiss (index in ordering o)    */
    /* material textures (map_Kd), resampled to 512x512 as gpurt.cpp:158-198 does; sampled as the
       shaders sample VolumeTextureTextures (include/sppm_texture.h).  num_textures = 0: none.   */
    uint32_t num_textures;
    const uint8_t* textures;           /* [num_textures][512][512][4] RGBA8 (A unused)           */
    const int32_t* material_texture;   /* [num_materials] the material's texture or -1           */
} sppm_scene;

/* Camera as the eye pass consumes it (glslppm.cpp:259-273): TCamera after TCamera::Set. */
typedef struct sppm_camera {
    float origin[3];
    float u[3], v[3], w[3];
    float distance;
    uint32_t width, height;
} sppm_camera;

/* TCamera::Set (camera.cpp:4-18): look-at basis and distance = H / (2 tan(fov/2)). */
void sppm_camera_look_at(sppm_camera* cam, const float origin[3], const float lookat[3],
                         uint32_t width, uint32_t height, float fov_degrees);

/* ---- host-side scene construction (what mesh.cpp and bvh.cpp do in the reference) ------------- */
typedef struct sppm_mesh sppm_mesh; /* owns the arrays an sppm_scene points into */

/* TMesh::LoadOBJ (mesh.cpp:491-693): OBJ + MTL, triangles only, positions*scale+offset. */
int sppm_mesh_load_obj(const char* path, const float offset[3], float scale, sppm_mesh** out);
/* Builds a mesh from flat arrays (positions [n][3][3], normals may be NULL -> face normals);
   materials as in sppm_material; light table derived like TMesh::PrepareLightSources. */
int sppm_mesh_from_arrays(uint32_t num_triangles, const float* positions, const float* normals,
                          const int32_t* material_ids, uint32_t num_materials,
                          const sppm_material* materials, sppm_mesh** out);
/* TBVH::Build (bvh.cpp:244-317): exact-SAH binary BVH, one triangle per leaf, 6 threaded
   orderings.  Stores the node arrays in the mesh. */
int sppm_mesh_build_bvh(sppm_mesh* mesh);
/* The same BVH arrays (node boxes and triangles, six threaded orderings with the reference's
   child-order rules) from a tree built on the GPU in milliseconds for multi-million-triangle
   meshes: Morton-ordered triangles clustered bottom-up (PLOC: mutual nearest neighbours by
   union-box area within a window of the cluster order), a tree close to a full SAH sweep's.  It
   differs from sppm_mesh_build_bvh's exact-SAH tree, so rays find the same closest triangle
   except at exact ties.  No counterpart in the reference (bvh.cpp builds on the host). */
int sppm_mesh_build_bvh_gpu(sppm_mesh* mesh, int device);
/* The GPU build with a chosen builder: SPPM_BVH_GPU_PLOC (the default above) or
   SPPM_BVH_GPU_LBVH, the linear BVH of a radix tree over the Morton codes (Karras 2012): faster
   to build, more nodes visited per ray. */
#define SPPM_BVH_GPU_PLOC 0
#define SPPM_BVH_GPU_LBVH 1
int sppm_mesh_build_bvh_gpu_ex(sppm_mesh* mesh, int device, int builder);
/* Fills *scene with pointers into the mesh (valid until sppm_mesh_destroy). */
int sppm_mesh_get_scene(const sppm_mesh* mesh, sppm_scene* scene);
void sppm_mesh_destroy(sppm_mesh* mesh);

/* ---- render context: one scene, one camera, one progressive state ------------------------------ */
typedef struct sppm_ctx sppm_ctx;

/* Allocates the per-pixel and per-photon state on `device` (CGPURT() + the texture and FBO set-up
   of main(), glslppm.cpp:691-795). */
int sppm_create(const sppm_config* cfg, int device, sppm_ctx** out);
/* Copies the scene to the device in the traversal layout (CGPURT::PrecalculateMeshData +
   CreateTextures, gpurt.cpp:8-16, 47-552). The caller's arrays are not retained. */
int sppm_upload_scene(sppm_ctx* ctx, const sppm_scene* scene);
/* Queues the camera's upload (the job descriptor, sppm_camera_upload_bytes() bytes, through a
   page-locked staging slot; the frames already queued keep the previous camera). */
int sppm_set_camera(sppm_ctx* ctx, const sppm_camera* cam);
size_t sppm_camera_upload_bytes(void);
/* Back to frame 0: re-seeds the random state (RandomizeTextures, glslppm.cpp:113-140). */
int sppm_reset(sppm_ctx* ctx);
/* Queues n SPPM frames (m_display, glslppm.cpp:214-536) on the context's stream. */
int sppm_run_passes(sppm_ctx* ctx, uint32_t n);
/* Waits for queued work; returns SPPM_ERR_WATCHDOG if a device loop bound was hit. */
int sppm_synchronize(sppm_ctx* ctx);

typedef enum sppm_image_kind {
    SPPM_IMAGE_RADIANCE = 0, /* linear L = tau / (R^2 pi Nemitted) + emission (re.fs:35-38)      */
    SPPM_IMAGE_DISPLAY = 1   /* 1 - exp(-60000 L), then sRGB (re.fs:41-47)                        */
} sppm_image_kind;
/* Resolves the image and copies width*height*3 floats (row 0 = bottom row, as GL) to rgb. */
int sppm_read_image(sppm_ctx* ctx, uint32_t kind, float* rgb, size_t num_floats);
/* The same without waiting (no counterpart in the reference, which displays every frame from
   the GPU): the resolve is queued behind the passes already queued, and the copy into rgb runs
   on a second stream beside the passes queued after it.  *ticket (numbered from 1) names the
   copy; rgb must stay valid and unread until sppm_image_wait(ctx, ticket) (or sppm_synchronize)
   returns.  Page-locked rgb (sppm_host_alloc) lets the copy overlap; with pageable memory the
   call waits for the copy.  At most 16 copies are in flight: a further call waits for the
   oldest. */
int sppm_read_image_async(sppm_ctx* ctx, uint32_t kind, float* rgb, size_t num_floats, uint64_t* ticket);
/* Waits until the copy named by ticket (and every older one) has ended. */
int sppm_image_wait(sppm_ctx* ctx, uint64_t ticket);
/* Sets *done to 1 when the copy named by ticket has ended, else 0; never waits. */
int sppm_image_query(sppm_ctx* ctx, uint64_t ticket, int* done);

/* Writes an image as sppm_read_image returns it to a file (no counterpart in the reference,
   which only displays):  SPPM_FILE_PFM keeps the linear floats (little-endian, bottom row first,
   as the format stores rows); SPPM_FILE_PPM writes binary 8-bit P6, top row first, with
   clamp(v, 0, 1) * 255 rounded -- meant for SPPM_IMAGE_DISPLAY images; SPPM_FILE_EXR writes an
   OpenEXR 2 single-part scanline file, uncompressed, channels B G R as 32-bit floats, top row
   first. */
typedef enum sppm_file_format { SPPM_FILE_PFM = 0, SPPM_FILE_PPM = 1, SPPM_FILE_EXR = 2 } sppm_file_format;
int sppm_write_image_file(const char* path, const float* rgb, uint32_t width, uint32_t height, uint32_t format);

/* Per-pixel / per-photon / per-slot state, for parity checks and checkpointing. */
typedef enum sppm_state_kind {
    SPPM_STATE_HIT_POSITION = 0,    /* float4/pixel  QueryPositionTexture (pos.xyz, dir.x)      */
    SPPM_STATE_HIT_REFLECTANCE = 1, /* float4/pixel  QueryReflectanceTexture (col, dir.y)       */
    SPPM_STATE_HIT_NORMAL = 2,      /* float4/pixel  QueryNormalTexture (nrm, dir.z)            */
    SPPM_STATE_EYE_RNG = 3,         /* float4/pixel  RandomEyeRayTexture                        */
    SPPM_STATE_HIT_TRIANGLE = 4,    /* int32/pixel   triangle of QueryIntersectionTexture, -1   */
    SPPM_STATE_EMISSION_N = 5,      /* float4/pixel  QueryEmissionPhotonCountTexture (emi, N)   */
    SPPM_STATE_FLUX_RADIUS = 6,     /* float4/pixel  QueryFluxRadiusTexture (tau, R)            */
    SPPM_STATE_PHOTON_POSITION = 7, /* float4/photon PhotonPositionTexture (pos, nrm.x)         */
    SPPM_STATE_PHOTON_FLUX = 8,     /* float4/photon PhotonFluxTexture (flux, nrm.y)            */
    SPPM_STATE_PHOTON_DIRECTION = 9,/* float4/photon PhotonDirectionTexture (dir, nrm.z)        */
    SPPM_STATE_PHOTON_RNG = 10,     /* float4/photon RandomPhotonTexture                        */
    SPPM_STATE_PHOTON_HIT = 11,     /* int32x2/photon (triangle or -1, path depth)              */
    SPPM_STATE_SLOT_WINNER = 12,    /* uint32/slot   photon id stored in the slot, 0xFFFFFFFF   */
    SPPM_STATE_SLOT_COUNT = 13,     /* uint32/slot   photons hashed to the slot                 */
    SPPM_STATE_HIT_T = 14,          /* float/pixel   t of QueryIntersectionTexture (.w)         */
    SPPM_STATE_STATS_N = 15,        /* double/pixel  N (mixed precision statistics)             */
    SPPM_STATE_STATS_R2 = 16,       /* double/pixel  R^2                                        */
    SPPM_STATE_STATS_TAU = 17       /* double3/pixel tau                                        */
} sppm_state_kind;
/* Copies one state array to host memory; `bytes` must equal the array's size.  The statistics
   (kinds 15-17) are held on the device as double-float pairs (two floats whose sum is the value)
   and arrive as doubles. */
int sppm_read_state(sppm_ctx* ctx, uint32_t kind, void* dst, size_t bytes);
/* Size in bytes of a state array (0 if the kind is not kept by this precision). */
size_t sppm_state_bytes(const sppm_ctx* ctx, uint32_t kind);

typedef struct sppm_frame_info {
    uint32_t frames;              /* FrameCount                                               */
    uint32_t eye_samples;         /* NumEyeSamples                                            */
    uint64_t photons_emitted;     /* NumPhotons, kept as an exact integer                     */
    float num_photons_f32;        /* NumPhotons as the reference accumulates it (float)        */
    float initial_radius;         /* InitialRadius of the last eye pass                        */
    float grid_scale;             /* GridScale                                                 */
    float bbox_min[3], bbox_max[3]; /* expanded hit-point bbox (BBMin/BBMax)                   */
    float aa_offset[2];           /* AAOffset of the last eye pass                             */
    uint64_t photon_segments;     /* photon ray segments traced so far                         */
    uint64_t eye_segments;        /* eye ray segments traced so far                            */
    uint64_t counted_segments;    /* photon segments traced while traversal counters were on   */
    uint64_t counted_nodes;       /* BVH nodes those segments visited                          */
    uint64_t counted_triangles;   /* triangles those segments tested                           */
    uint64_t coop_segments;       /* photon segments traced one per warp (a zero direction
                                     component, see sppm_debug_trace)                          */
    uint64_t kernel_launches;     /* kernels launched by sppm_run_passes since sppm_create      */
} sppm_frame_info;
int sppm_get_frame_info(sppm_ctx* ctx, sppm_frame_info* info);

/* Checkpoint / resume of the progressive state (no counterpart in the reference): a flat binary
   image of the frame counters, RNG states, hit points, photon records, hashed grid and
   progressive statistics -- not the scene or camera, which a resuming context uploads itself.
   The header records fingerprints of the scene (every array of the uploaded sppm_scene), of the
   camera and of the seed (seed_mode, seed).  Loading it into a context of the same image, photon
   and hash sizes, precision, seed, scene and camera continues the render exactly where it was
   saved (the next frames are bit-identical to an uninterrupted run); any other context rejects
   it with SPPM_ERR_ARG, naming what differs. */
size_t sppm_checkpoint_bytes(const sppm_ctx* ctx);
int sppm_save_checkpoint(sppm_ctx* ctx, void* dst, size_t bytes);
int sppm_load_checkpoint(sppm_ctx* ctx, const void* src, size_t bytes);
/* While enabled, the photon pass also counts BVH nodes visited and triangles tested (a separate
   kernel instantiation; results are unchanged).  Used for the algorithmic-byte roofline. */
int sppm_enable_traversal_counters(sppm_ctx* ctx, int enable);

/* Per-stage device time (ms) accumulated since the last call, measured with CUDA events on the
   context's stream around each stage launch; enable before the passes to be timed. */
typedef enum sppm_stage {
    SPPM_STAGE_FRAME_BEGIN = 0, /* hash clear + per-frame scalars                          */
    SPPM_STAGE_EYE = 1,         /* eyeraytrace.fs + max/min reductions                      */
    SPPM_STAGE_GRID = 2,        /* InitialRadius / GridScale (glslppm.cpp:294-311)          */
    SPPM_STAGE_PHOTON = 3,      /* photontrace.fs emit/bounce (+ trace, store, hash when fused) */
    SPPM_STAGE_GATHER = 4,      /* progressive.fs                                          */
    SPPM_STAGE_RESOLVE = 5,     /* re.fs                                                   */
    SPPM_STAGE_PHOTON_TRACE = 6, /* photon segment traversal (wavefront pass)              */
    SPPM_STAGE_PHOTON_STORE = 7, /* photon store + hash.fs/scatter/correction (wavefront)  */
    SPPM_STAGE_RAY_BINS = 8,     /* counting sort of the photon rays into bins (wavefront)  */
    SPPM_STAGE_PHOTON_SORT = 9,  /* counting-sort photon grid (SPPM_FLAG_PHOTON_GRID)        */
    SPPM_STAGE_COUNT = 10
} sppm_stage;
int sppm_enable_stage_timing(sppm_ctx* ctx, int enable);
/* Times only the stages whose bit (1 << stage) is set; 0 turns timing off. */
int sppm_set_stage_timing_mask(sppm_ctx* ctx, uint32_t mask);
int sppm_read_stage_times(sppm_ctx* ctx, float ms[SPPM_STAGE_COUNT], uint32_t launches[SPPM_STAGE_COUNT]);

/* Device time (ms) of `n` frames measured with CUDA events on the context's stream. */
int sppm_time_passes(sppm_ctx* ctx, uint32_t n, float* ms);

/* ---- launch shapes and their autotuner ------------------------------------------------------
   No counterpart in the reference (its shader passes are fixed draw calls).  The shapes change
   how a pass is launched, never what it computes: images and state are the same bit for bit under
   every tuning. */
typedef struct sppm_tuning {
    uint32_t trace_blocks_per_sm; /* resident blocks of the persistent photon traversal per SM
                                     (0 = as many as fit)                                       */
    uint32_t trace_refill_steps;  /* traversal steps a warp takes before it refills its idle
                                     lanes from the ray queue (0 = 32; 4-wide traversal 8)      */
    uint32_t eye_block;           /* threads per block of the eye pass (0 = 128; 32..128)       */
    uint32_t store_block;         /* of the photon store + hash insertion (0 = 128; 32..128)    */
    uint32_t gather_block;        /* of the gather + progressive update (0 = 256; 32..256)      */
    uint32_t unbinned_rays;       /* 1: photon rays traced in queue order instead of binned     */
    uint32_t trace_tail_lanes;    /* exact traversal: once the ray queue is drained, a warp with
                                     at most this many walking lanes hands those walks to a tail
                                     kernel that finishes each with all 32 lanes of a warp (the
                                     warp-cooperative walk; same results) (0 = off, up to 32)   */
    uint32_t wide_bvh;            /* plain FP32 path: 1 traces eye and photon rays through the
                                     4-wide quantised BVH (conservative slab tests, the exact
                                     triangle test, ties at equal t broken by the exact walk's
                                     order) instead of the binary threaded walk: fewer node
                                     fetches on large scenes, and the same hits except where the
                                     reference's own FP32 box test skips a box whose triangle is
                                     an ulp or two closer than the hit found so far
                                     (near-coincident triangles): the 4-wide walk then returns
                                     the closer triangle, so the state is no longer the
                                     reference's bit for bit (3 of 2M eye rays on a 4.1M-triangle
                                     mesh; none on the Cornell scenes).  The autotuner never sets
                                     it.  Ignored by the mixed path, which always uses it.       */
    uint32_t photon_wave;         /* wavefront queue depth: photon slots generated, binned,
                                     traced and stored per wave of the photon pass, so a wave's
                                     ray queue and photon records stay in L2 from one kernel to
                                     the next (0 = every slot in one wave; else >= 1024)         */
    uint32_t grid_cell_split;     /* counting-sort photon grid (SPPM_FLAG_PHOTON_GRID): grid cells
                                     per reference cell along each axis -- 1, 2, 4 or 8 (0 = 2);
                                     a hit point visits the cells its radius touches, so finer
                                     cells mean fewer photons visited and more cells looked up
                                     (same results)                                              */
} sppm_tuning;
/* Block sizes are multiples of 32.  The frame graphs are captured again with the new shapes. */
int sppm_set_tuning(sppm_ctx* ctx, const sppm_tuning* tuning);
/* The shapes in effect (defaults filled in). */
int sppm_get_tuning(sppm_ctx* ctx, sppm_tuning* tuning);
/* Runs the context's next passes under candidate shapes and leaves the fastest in effect:
   a grid over ray order x refill interval, then coordinate descent over the other fields (a
   second sweep over all of them when the first changed anything), each candidate run for one
   untimed and `cycles` timed eye-pass cycles
   (eye_pass_interval passes each), a candidate kept when it is at least 1 % faster than the best
   so far.  These are ordinary passes of the job (its frame count
   advances).  *best and *ms_per_pass (either may be NULL) receive the chosen shapes and their
   time per pass. */
int sppm_autotune(sppm_ctx* ctx, uint32_t cycles, sppm_tuning* best, float* ms_per_pass);
/* The hash-table size (hash load factor) by measurement: scratch contexts of this configuration,
   scene and camera with hash_slots = P, 2P and 4P (P = photon slots; load factors 1, 1/2, 1/4)
   each run `passes` untimed and `passes` timed passes; *hash_slots receives the fastest and
   ms_per_pass (may be NULL) the three times (-1 for a size above the 2^28-slot limit).  A table larger than P makes fewer grid cells share a
   slot, which changes the image: this is a configuration value chosen before a job starts. */
int sppm_tune_hash_slots(const sppm_config* cfg, const sppm_scene* scene, const sppm_camera* cam, int device,
                         uint32_t passes, uint32_t* hash_slots, float ms_per_pass[3]);

void sppm_destroy(sppm_ctx* ctx);

/* ---- stage-level entry points (device pointers) --------------------------------------------- */
/* The hash build of hash.fs + scatter.vs + correction.vs on caller-owned device arrays:
   for photon i (row-major in a photon_width-wide buffer) with flux[i].x >= 0, slot = hash of
   the grid cell floor((pos[i]-bbox_min)*grid_scale); count[slot] += 1; winner[slot] =
   min i unless the GL depth clip removes photon i.  pos/flux are float4 arrays (xyz used).
   winner/count (hash_slots entries each) are overwritten. Runs on `stream` (cudaStream_t). */
int sppm_hash_build(const float* d_pos, const float* d_flux, uint32_t photon_width,
                    uint32_t photon_height, uint32_t hash_slots, const float bbox_min[3],
                    float grid_scale, uint32_t flags, uint32_t* d_winner, uint32_t* d_count,
                    void* stream);

typedef enum sppm_reduce_op { SPPM_REDUCE_MIN = 0, SPPM_REDUCE_MAX = 1, SPPM_REDUCE_SUM = 2 } sppm_reduce_op;
/* ReduceTexture (glslppm.cpp:170-209) with min.fs / max.fs / sum.fs on a caller's device texture:
   d_texture holds resolution x resolution float4 texels, row 0 first (16-byte aligned), resolution
   a power of two in [2, 16384].  The texture is folded 2x2 level by level in the order of the
   reference's ping-pong draws, so min, max and sums are bit-identical to it; the 1x1 result is in
   out[4] (host memory) when the call returns.  Scratch: a (resolution/2)^2 float4 ping-pong buffer,
   allocated stream-ordered on `stream` (cudaStream_t, 0 = default stream) and freed before the call
   returns; the call synchronizes `stream`. */
int sppm_reduce_texture(const float* d_texture, uint32_t resolution, uint32_t op, float out[4], void* stream);

/* sppm_reduce_texture for callers that must not allocate device memory -- an engine that reserved
   the GPU's memory for its own allocator before loading this library, a render loop that forbids
   allocation (and the implicit synchronization cudaMalloc may bring) once it is running.  It has
   no counterpart in the reference, whose ReduceTexture draws into a texture created at start-up.
   Its scratch is a fixed 4 MiB array in the library's device memory, which every GPU that loads the
   library keeps until the process exits; resolutions above SPPM_REDUCE_NOALLOC_MAX_RESOLUTION are
   rejected with SPPM_ERR_ARG.  The first call on a device looks up the array's device address
   (cudaGetSymbolAddress, which may load the library's device code) and caches it for the device's
   current CUDA context; after a device reset (cudaDeviceReset) the next call sees a new context
   and looks the address up again.  Make the first call on a device, and the first after a reset,
   before any stream capture.  All calls share the array: calls that overlap on the GPU (on different
   streams, or from several threads) race on it and must be serialised by the caller.  Nothing in
   the array needs to start at zero.  Results equal sppm_reduce_texture's bit for bit. */
#define SPPM_REDUCE_NOALLOC_MAX_RESOLUTION 1024u
int sppm_reduce_texture_noalloc(const float* d_texture, uint32_t resolution, uint32_t op, float out[4],
                                void* stream);

/* ---- diagnostics ------------------------------------------------------------------------------ */
/* Message of the last failed call on this thread; returns the full message length. */
size_t sppm_last_error(char* buf, size_t buf_size);
/* Runs the pinned FP32 functions of sppm_fpmath.h on the GPU: fn 0 sin, 1 cos, 2 pow(x,y),
   3 exp, 4 log2, 5 exp2.  x, y, out are host arrays of n floats. */
int sppm_debug_fpmath(int fn, const float* x, const float* y, float* out, size_t n);
/* Traces n single rays (org, dir: 3 floats each, host arrays) through the uploaded scene's exact
   FP32 traversal (raytrace() of photontrace.fs:123-255 when photon != 0, of eyeraytrace.fs:67-290
   with back-face culling when cull != 0 otherwise): tri[i] = closest triangle or -1, t[i] = its
   t (the initial bound when nothing is hit).  mode 0 traces one ray per thread, mode 1 one ray
   per warp, mode 2 one ray per block of 1024 threads (the form the photon pass uses for rays
   with a zero direction component); all give the same result.  Mode 3 traces the mixed
   path's 4-wide quantised BVH instead (contexts of SPPM_PRECISION_MIXED, or any context whose scene
   has the 4-wide tree): its triangle and t equal the exact traversal's, ties at equal t included
   (broken by each triangle's leaf position in the ray's ordering), except where the exact
   traversal's rounded box test skips a box whose triangle is closer: mode 3 returns that closer
   triangle. */
int sppm_debug_trace(sppm_ctx* ctx, const float* org, const float* dir, size_t n, int photon, int cull, int mode,
                     int32_t* tri, float* t);
/* The photon rays the last pass traced (the wavefront's ray queue; not with
   SPPM_FLAG_FUSED_PHOTON): *count rays, origin and direction (3 floats each) and the photon slot
   each belongs to.  With org, dir and photon all null only *count is set.  For tests that trace
   the same rays again through sppm_debug_trace. */
int sppm_debug_photon_rays(sppm_ctx* ctx, float* org, float* dir, uint32_t* photon, size_t capacity, size_t* count);
/* The counting-sort photon grid of the last pass (contexts with SPPM_FLAG_PHOTON_GRID): offsets
   [hash_slots + 1] (the records of slot s are offsets[s] .. offsets[s+1]-1) and records [4 words
   per stored photon] in slot order; *num_records = offsets[hash_slots].  Word 0-1: the position as
   three 21-bit unsigned fixed-point grid coordinates (x | y << 21 | z << 42 of a 64-bit word, low
   word first; coordinate = floor((p - bbox_min) * grid_scale * 2^F) with F = 21 - bits(cells + 1),
   cells = the grid's largest cell count along an axis; all ones: outside the grid); word 2: flux
   r | g << 16 (FP16, scaled by 1 / (light area * 3.141592)); word 3: flux b | direction << 16
   (octahedral, two signed 8-bit components).  Within a slot the order of the records is not
   fixed.  With offsets and records null only *num_records is set. */
int sppm_debug_photon_grid(sppm_ctx* ctx, uint32_t* offsets, size_t offsets_capacity, uint32_t* records,
                           size_t records_capacity, uint32_t* num_records);
/* The order the photon traversal takes the ray bins in (contexts with binned rays).  A ray's bin
   is its direction class (cube face of the direction x the signs of its two minor components,
   24) x its origin cell (8^3 cells of the scene's bounding sphere, Morton-ordered): bin =
   class * 512 + cell.  rank[bin] = the bin's position in the traversal order; cost[position] =
   (node steps << 32) + rays of the walks traced since the last reorder.  At the start of a frame
   with an eye pass that begins 8 or more frames after the last reorder the bins are reordered: by descending mean steps per ray (the mean m
   quantised to 1 + min(254, m < 128 ? m : 128 + (m - 128) / 8), bins without rays last), equal
   keys in bin order, and the costs restart from zero; the first frames use bin order.  The order
   never changes a result.  capacity = entries of each array (at least *num_bins; with rank and
   cost null only *num_bins is set). */
int sppm_debug_ray_bins(sppm_ctx* ctx, uint32_t* rank, uint64_t* cost, size_t capacity, uint32_t* num_bins);
/* Page-locked host memory (cudaMallocHost) for the host buffers of sppm_read_image and friends:
   copies to it run at the interconnect's DMA rate instead of being staged through the driver. */
int sppm_host_alloc(size_t bytes, void** ptr);
void sppm_host_free(void* ptr);
/* Number of CUDA devices (0 when none); never fails. */
int sppm_device_count(void);
uint32_t sppm_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SPPM_H */

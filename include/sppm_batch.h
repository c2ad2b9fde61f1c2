/* Batched SPPM: many render jobs -- each with its own scene, camera, image size and photon
 * budget -- advanced together, every stage of a pass being ONE launch over all jobs.
 *
 * No counterpart in the reference: glslppm renders one scene per process (CGPURT, gpurt.h:29-67,
 * driven by m_display, glslppm.cpp:214-536).  A batch job follows exactly the single-job pass
 * sequence of sppm.h; a job's state after n passes in a batch is the same as after n passes of
 * a single-job context with the same configuration, scene and camera.
 *
 * Jobs are admitted against a device-memory budget (sppm_batch_job_bytes gives a job's
 * footprint) and keep their scene, hit points and progressive state resident until removed.
 * Passes are queued on the batch's stream as one CUDA graph per eye-pass phase.  All calls on
 * one batch must come from one host thread at a time. */
#ifndef SPPM_BATCH_H
#define SPPM_BATCH_H

#include "sppm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sppm_batch sppm_batch;

typedef struct sppm_batch_config {
    uint32_t precision;         /* SPPM_PRECISION_* of every job                               */
    uint32_t flags;             /* SPPM_FLAG_UNBINNED_RAYS, SPPM_FLAG_EAGER_LAUNCH,
                                   SPPM_FLAG_FUSED_PHOTON (the job flags stay per job)         */
    uint32_t eye_pass_interval; /* shared by every job (MaxNumberOfBounces)                    */
    uint32_t max_jobs;          /* job slots (job ids are 0 .. max_jobs-1)                     */
    uint64_t memory_budget;     /* device bytes jobs may hold; 0 = 90% of the free memory
                                   when the batch is created                                   */
} sppm_batch_config;

typedef struct sppm_batch_info {
    uint32_t num_jobs;          /* jobs resident                                               */
    uint32_t max_jobs;
    uint64_t bytes_used;        /* device bytes of the jobs, launch tables and ray queue       */
    uint64_t memory_budget;
    uint64_t frames;            /* passes queued since creation                                */
    uint64_t kernel_launches;   /* kernels launched by sppm_batch_run_passes                   */
    uint64_t photon_slots;      /* photon slots per pass over all jobs                         */
    uint64_t pixels;            /* pixels over all jobs                                        */
} sppm_batch_info;

void sppm_batch_config_defaults(sppm_batch_config* cfg);
int sppm_batch_create(const sppm_batch_config* cfg, int device, sppm_batch** out);
void sppm_batch_destroy(sppm_batch* b);

/* Device bytes a job with this configuration and scene holds in the batch (state + scene +
   its share of the ray queue). */
int sppm_batch_job_bytes(const sppm_batch* b, const sppm_config* cfg, const sppm_scene* scene, uint64_t* bytes);
/* Uploads the scene and camera, seeds the job's state and admits it: SPPM_ERR_OOM when the
   budget (or the device) has no room, SPPM_ERR_STATE when every slot is taken.  The job's first
   pass is the batch's next pass. */
int sppm_batch_add_job(sppm_batch* b, const sppm_config* cfg, const sppm_scene* scene, const sppm_camera* cam,
                       uint32_t* job);

/* Scenes prepared ahead of time.  Adding a job does host work before its copies to the device:
   the traversal layout of the six node orderings, the 4-wide tree with its leaf ranks, a
   fingerprint of every array (the reference's CGPURT::CreateTextures, gpurt.cpp:47-552, does the
   same packing in the frame loop's thread).  sppm_scene_prepare does that work on the calling
   thread -- any thread, e.g. while the batch renders -- and sppm_batch_add_job_prepared then only
   allocates and copies: the same job as sppm_batch_add_job.  A prepared scene owns its arrays
   (the source may be freed once it returns) and may be added to any number of jobs. */
typedef struct sppm_prepared_scene sppm_prepared_scene;
int sppm_scene_prepare(const sppm_scene* scene, sppm_prepared_scene** out);
void sppm_scene_prepared_destroy(sppm_prepared_scene* scene);
/* sppm_batch_job_bytes for a prepared scene (its scene arena exactly). */
int sppm_batch_job_bytes_prepared(const sppm_batch* b, const sppm_config* cfg, const sppm_prepared_scene* scene,
                                  uint64_t* bytes);
/* A job's seeded random-state tables (the host-side fill of RandomizeTextures, glslppm.cpp:77-140,
   for this configuration's image, photon buffer, seed and seed mode), made ahead of time on the
   calling thread. */
typedef struct sppm_prepared_state sppm_prepared_state;
int sppm_state_prepare(const sppm_config* cfg, sppm_prepared_state** out);
void sppm_state_prepared_destroy(sppm_prepared_state* state);
/* sppm_batch_add_job with a prepared scene and, when state is not NULL, prepared tables (of the
   same configuration: SPPM_ERR_ARG otherwise); the job is the same. */
int sppm_batch_add_job_prepared(sppm_batch* b, const sppm_config* cfg, const sppm_prepared_scene* scene,
                                const sppm_prepared_state* state, const sppm_camera* cam, uint32_t* job);
int sppm_batch_remove_job(sppm_batch* b, uint32_t job);
int sppm_batch_reset_job(sppm_batch* b, uint32_t job);
int sppm_batch_set_camera(sppm_batch* b, uint32_t job, const sppm_camera* cam);
/* The same as sppm_batch_set_camera(b, jobs[i], &cams[i]) for i in [0, n), with the n descriptor
   uploads queued as one launch (per 128 jobs) instead of n.  Every id is checked before any
   camera changes: an unknown or repeated id fails the whole call with SPPM_ERR_ARG. */
int sppm_batch_set_cameras(sppm_batch* b, uint32_t n, const uint32_t* jobs, const sppm_camera* cams);

/* Queues n passes of every resident job. */
int sppm_batch_run_passes(sppm_batch* b, uint32_t n);
/* Launch shapes of the batch's passes (sppm_tuning in sppm.h; one set for all jobs) and their
   autotuner, which runs the batch's next passes as sppm_autotune does a context's. */
int sppm_batch_set_tuning(sppm_batch* b, const sppm_tuning* tuning);
int sppm_batch_get_tuning(sppm_batch* b, sppm_tuning* tuning);
int sppm_batch_autotune(sppm_batch* b, uint32_t cycles, sppm_tuning* best, float* ms_per_pass);
int sppm_batch_time_passes(sppm_batch* b, uint32_t n, float* ms);
int sppm_batch_synchronize(sppm_batch* b);

int sppm_batch_read_image(sppm_batch* b, uint32_t job, uint32_t kind, float* rgb, size_t num_floats);
/* sppm_read_image_async / sppm_image_wait / sppm_image_query for one job of the batch (the
   tickets are the batch's; a removed job's copy is waited for before its memory is freed). */
int sppm_batch_read_image_async(sppm_batch* b, uint32_t job, uint32_t kind, float* rgb, size_t num_floats,
                                uint64_t* ticket);
int sppm_batch_image_wait(sppm_batch* b, uint64_t ticket);
int sppm_batch_image_query(sppm_batch* b, uint64_t ticket, int* done);
size_t sppm_batch_state_bytes(const sppm_batch* b, uint32_t job, uint32_t kind);
int sppm_batch_read_state(sppm_batch* b, uint32_t job, uint32_t kind, void* dst, size_t bytes);
int sppm_batch_get_frame_info(sppm_batch* b, uint32_t job, sppm_frame_info* info);
/* sppm_batch_get_frame_info for n jobs at once (one device-to-host copy for all of them, of
   sppm_batch_frame_record_bytes() bytes per job). */
int sppm_batch_get_frame_infos(sppm_batch* b, const uint32_t* jobs, uint32_t n, sppm_frame_info* infos);
size_t sppm_batch_frame_record_bytes(void);
int sppm_batch_get_info(sppm_batch* b, sppm_batch_info* info);
/* Checkpoints of one job (the layout of sppm_save_checkpoint): a job can move between a batch
   and a single-job context, or be preempted and resumed. */
size_t sppm_batch_checkpoint_bytes(const sppm_batch* b, uint32_t job);
int sppm_batch_save_checkpoint(sppm_batch* b, uint32_t job, void* dst, size_t bytes);
int sppm_batch_load_checkpoint(sppm_batch* b, uint32_t job, const void* src, size_t bytes);

int sppm_batch_set_stage_timing_mask(sppm_batch* b, uint32_t mask);
int sppm_batch_read_stage_times(sppm_batch* b, float ms[SPPM_STAGE_COUNT], uint32_t launches[SPPM_STAGE_COUNT]);
int sppm_batch_enable_traversal_counters(sppm_batch* b, int enable);

#ifdef __cplusplus
}
#endif
#endif /* SPPM_BATCH_H */

/* SPPM render server: continuous batching of render requests on one GPU.
 *
 * No counterpart in the reference (glslppm renders one scene interactively).  A server owns a
 * batch (sppm_batch.h) and one host thread that loops: admit waiting requests in arrival order
 * while the batch has a free slot and its memory budget has room for the request's footprint;
 * queue passes of every resident job (one launch per stage over all of them); retire the jobs
 * that reached their target pass count (read the radiance image back, free the job's device
 * memory).  Requests that arrive while others are on the GPU join the batch at the next pass, so
 * their work overlaps.  A job's result equals the single-job context's after the same number of
 * passes, whatever else is in the batch.
 *
 * submit copies the scene, so the caller's arrays may be freed on return.  poll, wait,
 * fetch_image and get_stats may be called from any thread. */
#ifndef SPPM_SERVER_H
#define SPPM_SERVER_H

#include "sppm_batch.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sppm_server sppm_server;

typedef enum sppm_request_state {
    SPPM_REQUEST_QUEUED = 0,   /* waiting for a slot and memory                               */
    SPPM_REQUEST_RUNNING = 1,  /* resident in the batch                                        */
    SPPM_REQUEST_DONE = 2,     /* target passes reached; image ready for sppm_server_fetch_image */
    SPPM_REQUEST_FAILED = 3    /* rejected or failed; status holds the sppm_status             */
} sppm_request_state;

typedef struct sppm_server_config {
    sppm_batch_config batch;   /* precision, flags, eye-pass interval, job slots, memory budget */
    uint32_t passes_per_step;  /* passes queued between admission/retirement rounds (>= 1)     */
    uint32_t max_queue;        /* requests waiting for admission before submit refuses         */
    sppm_tuning tuning;        /* launch shapes of the server's batch (sppm.h; zeros: defaults) */
} sppm_server_config;

typedef struct sppm_request_info {
    uint32_t state;            /* sppm_request_state                                           */
    int32_t status;            /* sppm_status of a failed request, else 0                      */
    uint32_t passes_done;      /* passes queued for the job so far                             */
    uint32_t target_passes;
    uint32_t width, height;
    uint64_t photons_emitted;  /* when done                                                    */
    double t_submit, t_admit, t_done;  /* seconds since the server was created (0 = not yet)   */
} sppm_request_info;

typedef struct sppm_server_stats {
    uint64_t submitted, admitted, completed, failed;
    uint32_t resident, queued;
    uint64_t bytes_used, memory_budget;
    uint64_t passes;           /* batch passes queued                                          */
    uint64_t photons;          /* photons emitted by completed requests                        */
    double busy_seconds;       /* wall time with at least one resident job                     */
} sppm_server_stats;

void sppm_server_config_defaults(sppm_server_config* cfg);
int sppm_server_create(const sppm_server_config* cfg, int device, sppm_server** out);
/* Stops the loop (jobs still resident are dropped) and frees everything. */
void sppm_server_destroy(sppm_server* s);

/* Queues a request of target_passes passes; SPPM_ERR_OOM when its footprint exceeds the whole
   budget, SPPM_ERR_STATE when max_queue requests are waiting. */
int sppm_server_submit(sppm_server* s, const sppm_config* cfg, const sppm_scene* scene, const sppm_camera* cam,
                       uint32_t target_passes, uint64_t* ticket);
int sppm_server_poll(sppm_server* s, uint64_t ticket, sppm_request_info* info);
/* Waits until the request is done or failed, or timeout_seconds pass (SPPM_ERR_STATE). */
int sppm_server_wait(sppm_server* s, uint64_t ticket, double timeout_seconds, sppm_request_info* info);
/* Copies a done request's linear radiance image (width*height*3 floats) and forgets the request. */
int sppm_server_fetch_image(sppm_server* s, uint64_t ticket, float* rgb, size_t num_floats);
int sppm_server_get_stats(sppm_server* s, sppm_server_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* SPPM_SERVER_H */

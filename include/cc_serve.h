/*
 * cc_serve.h - a continuous-batching CC server on one GPU (libccgpu.so).
 *
 * No counterpart in the reference (one graph per driver run).  Clients submit
 * graphs as they arrive; a worker thread admits them while the HBM budget
 * allows (the rest wait on the host in arrival order), copies them to the
 * device on a copy stream, and whenever a compute stream is free it
 * coalesces every staged request into one batched launch: graphs up to the
 * shared-memory size are solved one CTA each, larger ones by the grid-wide
 * hook-and-compress on the same stream.  New requests are admitted and
 * copied while earlier batches run.  Labels stay on the device until the
 * client collects them (cc_serve_wait / cc_serve_poll), which frees the
 * request's memory and budget.  Each request's labels are the canonical
 * labels cc_gpu_run would give that graph alone.
 *
 * The host arrays of a submitted graph must stay valid until its labels have
 * been collected.
 */
#ifndef CC_SERVE_H_
#define CC_SERVE_H_

#include "cc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cc_server cc_server;

typedef struct cc_serve_config {
  uint64_t hbm_budget_bytes;   /* device bytes requests may hold (default 120 GB) */
  uint32_t max_batch_graphs;   /* graphs coalesced into one launch (default 1024) */
  uint32_t compute_streams;    /* batches in flight at once (default 4) */
  uint32_t smem_max_n;         /* graphs up to this many vertices (and 32768 entries) go one
                                  CTA each (default 16384) */
  uint32_t batch_window_us;    /* a free stream waits up to this long after the oldest staged
                                  request for more to coalesce, unless the batch is full
                                  (default 0: launch at once) */
} cc_serve_config;

typedef struct cc_serve_ticket_info {
  double submit_s;    /* host clock (seconds) at submit */
  double admit_s;     /* admitted under the budget, copy enqueued */
  double done_s;      /* labels ready on the device */
  uint32_t batch_id;  /* launch the request rode in */
  uint32_t batch_size;
} cc_serve_ticket_info;

typedef struct cc_serve_stats {
  uint64_t submitted, completed, collected;
  uint64_t batches;            /* coalesced launches */
  uint64_t bytes_in_use;       /* device bytes held by admitted requests */
  uint64_t peak_bytes_in_use;
  uint64_t waiting;            /* requests not yet admitted */
} cc_serve_stats;

void cc_serve_config_default(cc_serve_config *c);
int cc_serve_create(cc_server **out, int device, const cc_serve_config *c);
/* Destroys after draining in-flight work; uncollected results are dropped. */
int cc_serve_destroy(cc_server *s);
/* Submit a graph (host CSR, uint32 or uint64 ids; num_parts is ignored).
   CC_ERR_BUSY: the graph alone exceeds the budget. */
int cc_serve_submit(cc_server *s, const cc_csr *g, uint64_t *ticket);
/* Non-blocking collect: *done = 1 and labels_out (n x id_bytes, host) filled
   when the labels are ready; the ticket is then retired.  info may be NULL. */
int cc_serve_poll(cc_server *s, uint64_t ticket, void *labels_out, int *done,
                  cc_serve_ticket_info *info);
/* Blocking collect, with a timeout in seconds (<= 0: wait forever);
   CC_ERR_TIMEOUT when it runs out (the ticket stays valid). */
int cc_serve_wait(cc_server *s, uint64_t ticket, void *labels_out, double timeout_s,
                  cc_serve_ticket_info *info);
int cc_serve_get_stats(cc_server *s, cc_serve_stats *out);
/* Host clock used by the timestamps (seconds, monotonic). */
double cc_serve_now(void);

#ifdef __cplusplus
}
#endif

#endif /* CC_SERVE_H_ */

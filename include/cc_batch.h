/*
 * cc_batch.h - many independent graphs in one solve (libccgpu.so).
 *
 * No counterpart in the reference, which solves one distributed graph per
 * driver run (app/exp_contraction.cpp:75-105).  The graphs are packed into one
 * segmented CSR: graph i owns vertices [voff[i], voff[i+1]) of a global row
 * offset array and stores LOCAL neighbour ids (0 .. n_i - 1).  Labels come
 * back as local canonical labels: the minimum local id of each vertex's
 * component inside its own graph, i.e. exactly what cc_gpu_run() returns for
 * that graph alone.
 *
 * One solve runs a small fixed number of launches for all graphs: graphs up
 * to a tuned size are solved whole by one CTA each in shared memory; larger
 * graphs share a grid-wide sampled linking (two neighbours per vertex, then
 * only the rows outside each graph's largest component).  The schedule (CTA size,
 * shared-memory size bucket, vertex- or edge-parallel hooking) comes from a
 * cc_batch_tuning that cc_batch_autotune() measures per size bucket.
 */
#ifndef CC_BATCH_H_
#define CC_BATCH_H_

#include "cc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cc_batch {
  uint32_t k;               /* number of graphs */
  uint32_t where;           /* CC_HOST or CC_DEVICE for every array below */
  uint64_t total_n;         /* sum of n_i */
  uint64_t total_m;         /* sum of directed entries */
  const uint64_t *voff;     /* k+1 vertex offsets */
  const uint64_t *row_ptr;  /* total_n+1 offsets into col (global positions) */
  const uint32_t *col;      /* total_m LOCAL neighbour ids */
} cc_batch;

/* Schedule of the batched solve, one entry per size bucket. */
#define CC_BATCH_BUCKETS 4
typedef struct cc_batch_tuning {
  uint32_t smem_max_n[CC_BATCH_BUCKETS];  /* bucket b holds graphs with n <= smem_max_n[b]
                                             (increasing; 0 = unused); larger graphs
                                             go to the grid-wide path */
  uint32_t threads[CC_BATCH_BUCKETS];     /* CTA size of bucket b */
  uint32_t edge_parallel[CC_BATCH_BUCKETS]; /* 1: threads stride over edges, 0: over vertices */
  uint32_t hub_degree;                     /* grid-wide path: rows above (outside the largest
                                             component) go one warp per row */
  uint32_t use_graph;                      /* replay the launches as one CUDA graph */
} cc_batch_tuning;

/* Default schedule (used when tuning is NULL). */
void cc_batch_tuning_default(cc_batch_tuning *t);

/* Solve every graph of *b; labels_out has total_n uint32 entries and lives
   where labels_where says.  algo must be CC_EXP or CC_ALLREDUCE (one rank per
   graph: both reduce to the hook-and-compress solve); other options go
   through cc_gpu_run per graph. */
int cc_batch_run(cc_ctx *ctx, const cc_batch *b, const cc_batch_tuning *tuning,
                 uint32_t *labels_out, uint32_t labels_where);

/* The plain path that the batched solve is measured against: one
   cc_ctx_run(algo, one rank) per graph, looped in C++ on ctx's stream (each
   solve ends with its stream synchronisation, as a caller solving the graphs
   one by one would see).  Device arrays only; labels_out: total_n uint32 on
   the device.  Before the loop one kernel writes per-graph row offsets that
   start at 0 (held by ctx for the next call).  The per-graph loop of the
   reference's drivers (app/exp_contraction.cpp:75-155) has this shape. */
int cc_batch_run_plain(cc_ctx *ctx, const cc_batch *b, cc_algo algo, const cc_config *cfg,
                       uint64_t seed, uint32_t *labels_out);

/* Time candidate schedules on *b (device arrays) and write the fastest per
   size bucket to *out.  reps: timed repetitions per candidate. */
int cc_batch_autotune(cc_ctx *ctx, const cc_batch *b, int reps, cc_batch_tuning *out);

#ifdef __cplusplus
}
#endif

#endif /* CC_BATCH_H_ */

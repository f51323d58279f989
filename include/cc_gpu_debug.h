/*
 * cc_gpu_debug.h - test hooks of libccgpu: single stages of the solve, run on
 * the calling thread's default context.  They exist so that each kernel can
 * be checked on its own against the CPU oracle; they are not part of the
 * drop-in boundary and have no counterpart in the reference.  All pointers
 * are device pointers unless stated; graphs must have uint32 ids where noted.
 */
#ifndef CC_GPU_DEBUG_H_
#define CC_GPU_DEBUG_H_

#include "cc_gpu.h"
#include "cc_serve.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Deviate threshold table for beta into host array out (cap entries);
   returns its length. */
int cc_debug_geo_table(double beta, uint64_t *out, int cap);
/* The counter-based hash behind every variate (host evaluation). */
uint64_t cc_debug_hash3(uint64_t seed, uint64_t a, uint64_t b);
/* Exponential-shift decomposition of a uint32 device graph: cluster_out[i] =
   index of i's centre.  vid: original id of each vertex (device). */
int cc_debug_ldd(const cc_csr *g, const uint32_t *vid, uint64_t seed, uint32_t level,
                 double beta, int gated, uint32_t *cluster_out, uint32_t *rounds_out);
/* Local-contraction sweeps: cluster_out[i] = index of the minimum key in the
   two-hop closed neighbourhood of i. */
int cc_debug_local_sweeps(const cc_csr *g, const uint32_t *vid, uint64_t seed, uint32_t level,
                          uint32_t *cluster_out);
/* Quotient graph of g under cl (cluster ids < ncl).  cut_parts > 0 keeps only
   edges between different virtual ranks.  Outputs are device buffers sized
   rp_out: ncl+1, col_out: g->m_dir, vid_out: ncl, newid_out: ncl. */
int cc_debug_contract(const cc_csr *g, const uint32_t *cl, uint64_t ncl,
                      const uint32_t *vid_of_cluster, uint32_t cut_parts, uint64_t *rp_out,
                      uint32_t *col_out, uint32_t *vid_out, uint32_t *newid_out,
                      uint64_t *n_out, uint64_t *m_out);
/* Partition-local components (g->num_parts ranks): labels_out[v] = minimum id
   of v's local component (uint32, device). */
int cc_debug_local_components(const cc_csr *g, uint32_t *labels_out);
/* Stable radix sort of n device uint64 keys on bits [0, bits). */
int cc_debug_radix_sort(uint64_t *keys, uint64_t n, int bits);
/* Test hook: caps every iterative round loop of ctx's solves (decomposition,
   label and shortcut propagation) at `cap` rounds (0 restores the default
   n + 2), so that a test reaches CC_ERR_NO_CONVERGENCE without a faulty
   kernel; the context stays usable. */
int cc_debug_set_round_cap(cc_ctx *ctx, uint32_t cap);
/* Test hook: the next request submitted to s fails on purpose at `where`
   (1: staging, as if its device allocation failed - collect returns
   CC_ERR_OOM; 2: its launch, as if a launch failed - collect returns
   CC_ERR_CUDA; use a graph above the one-CTA size for 2, a failed one-CTA
   launch fails every small request of that launch).  0 cancels. */
int cc_serve_debug_fail_next(cc_server *s, int where);
/* Shortcut propagation on a uint32 device graph from the given labels. */
int cc_debug_shortcut(const cc_csr *g, uint32_t *labels_inout, uint32_t hitters,
                      uint32_t *rounds_out);

#ifdef __cplusplus
}
#endif

#endif /* CC_GPU_DEBUG_H_ */

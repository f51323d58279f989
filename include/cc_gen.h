/*
 * cc_gen.h - seeded synthetic graph generators (libccgen.so, host C++).
 *
 * The reference takes its inputs from KaGen (github.com/sebalamm/KaGen, an
 * empty submodule in the reference tree) through IOUtility::LoadGraph
 * (lib/io/io_utils.h:59-83: gnm_undirected, grid_2d, rhg, ...).  These
 * generators produce the same graph families with the same parameters as
 * symmetric CSR, from a counter-based hash of (seed, index), so every host
 * builds the same graph for the same arguments.  Self-loops and duplicate
 * edges are dropped; adjacency rows are sorted.
 */
#ifndef CC_GEN_H_
#define CC_GEN_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cc_host_graph {
  uint64_t n;         /* vertices */
  uint64_t m_dir;     /* directed entries */
  uint64_t *row_ptr;  /* n+1, malloc'ed */
  void *col;          /* m_dir ids of id_bytes each, malloc'ed */
  uint32_t id_bytes;  /* 4 or 8 */
  uint32_t pad_;
} cc_host_graph;

/* Erdos-Renyi G(n, m): m endpoint pairs drawn uniformly (gnm_undirected). */
int cc_gen_gnm(uint64_t n, uint64_t m, uint64_t seed, uint32_t id_bytes, cc_host_graph *out);

/* 2D bond percolation on an X x Y lattice (grid_2d with -p): vertex id
   y*X + x, each right/down lattice edge kept independently with
   probability p; not periodic. */
int cc_gen_grid(uint64_t X, uint64_t Y, double p, uint64_t seed, uint32_t id_bytes,
                cc_host_graph *out);

/* Random hyperbolic graph, threshold model (rhg): n points in a disk of
   radius R, radial density alpha sinh(alpha r) with alpha = (gamma-1)/2,
   edge iff hyperbolic distance <= R; R chosen for the expected average
   degree avg_deg.  Vertex ids follow the angular order. */
int cc_gen_rhg(uint64_t n, double avg_deg, double gamma, uint64_t seed, uint32_t id_bytes,
               cc_host_graph *out);
/* The disk radius R that cc_gen_rhg uses for (n, avg_deg, gamma). */
double cc_gen_rhg_radius(uint64_t n, double avg_deg, double gamma);
/* Test aid: the number of vertex pairs on which g (a cc_gen_rhg result for the
   same arguments) disagrees with the model's edge test applied to every pair,
   O(n^2); ~0 for bad arguments. */
uint64_t cc_gen_rhg_verify(uint64_t n, double avg_deg, double gamma, uint64_t seed,
                           const cc_host_graph *g);

void cc_host_graph_free(cc_host_graph *g);

/* k independent G(n_i, m_i) graphs packed as a segmented CSR (cc_batch.h
   layout: global row offsets, LOCAL uint32 neighbour ids).  Graph i draws
   log2 n_i ~ U[log2_nmin, log2_nmax], average degree d_i ~ U[dmin, dmax],
   m_i = round(n_i d_i / 2) endpoint pairs, all from hash(seed, i). */
typedef struct cc_host_batch {
  uint32_t k;
  uint32_t pad_;
  uint64_t total_n, total_m;
  uint64_t *voff;     /* k+1 */
  uint64_t *row_ptr;  /* total_n+1 */
  uint32_t *col;      /* total_m */
} cc_host_batch;

int cc_gen_batch(uint32_t k, double log2_nmin, double log2_nmax, double dmin, double dmax,
                 uint64_t seed, cc_host_batch *out);
void cc_host_batch_free(cc_host_batch *b);

/* Input files, as the reference drivers read them with -input (GraphIO,
   lib/io/graph_io.h): METIS text ("n m" header, one line of 1-based
   neighbours per vertex, '%' comments), the sorted edge file ("<type> n m"
   header, "e u w" records of 1-based endpoints) and the sorted binary file
   (uint64 n, uint64 m, m pairs of uint64 1-based endpoints).  The result is
   the symmetric CSR with sorted rows, self-loops and repeated edges dropped;
   a malformed file or an endpoint outside [1, n] gives CC_ERR_INVALID.  Free
   with cc_host_graph_free. */
int cc_read_metis(const char *path, uint32_t id_bytes, cc_host_graph *out);
int cc_read_edge_list(const char *path, uint32_t id_bytes, cc_host_graph *out);
int cc_read_binary_edges(const char *path, uint32_t id_bytes, cc_host_graph *out);

#ifdef __cplusplus
}
#endif

#endif /* CC_GEN_H_ */

// kernels.h - host-side launchers of the libccgpu kernels.
//
// Every launcher enqueues work on the given stream and adds its launch count
// and algorithmic bytes to a Counters record.  The byte formulas are those of
// the measurement contract: s_o = 8 (row offsets), s_i = id bytes, s_k = 8 (key
// or label word).
#pragma once

#include "common.cuh"

namespace ccg {

// A CSR graph on the device.  idb is 4 or 8 for the caller's input graph and
// 4 for every graph the library builds itself.
struct Csr {
  uint64_t n = 0, m = 0;
  const uint64_t *rp = nullptr;
  const void *col = nullptr;
  int idb = 4;
  int *err = nullptr;  // device error word for caller-provided graphs
};

// ---- union-find hook-and-compress (uf.cu) ---------------------------------
// parent[v] <- minimum vertex id of v's component.  With pm != nullptr only
// edges whose endpoints lie in the same virtual rank are used, so parent[v] is
// the minimum id of v's partition-local component
// (exponential_contraction.h:391-411 FindLocalComponents).
enum : int { kUfAuto = 0, kUfGlobal = 1, kUfTiled = 2, kUfSampled = 3 };
// The row-sample decisions of one graph, remembered by a context so that a
// graph solved again (same buffers, sizes and tuning) skips the sample and
// its host round trip.  The decisions only pick a schedule: every schedule
// gives the same labels, so a caller that rewrites a graph in place between
// solves gets correct labels either way.
struct UfDecisionCache {
  const void *rp = nullptr, *col = nullptr;
  uint64_t n = 0, m = 0, parts_key = 0;
  uint32_t tile = 0, hub = 0;
  bool valid = false;
  bool tiles = false, link_tiles = false, few_hubs = true;
};
struct UfTuning {
  int mode = kUfAuto;  // auto: tiled, global (L2-resident, few hubs) or sampled from a row sample
  uint32_t hub_degree = 32;      // rows above: split into pieces of 2048 edges
  uint32_t tile_vertices = 32768;  // vertices per CTA tile (2 bytes of shared memory each)
  uint32_t tile_threads = 1024;
  int link_tiles = -1;  // sampled linking: link rounds tiled (1) or global (0); -1 decide from a row sample
  UfDecisionCache *cache = nullptr;  // the context's; nullptr: sample every time
};
// Host source of a caller graph whose device buffers are still empty: the
// tiled pass copies tile-aligned chunks on `copy` and overlaps them with the
// tile kernel (rp/col of the Csr are the destination device buffers); read in
// place, rp/col of the Csr are the device addresses of the caller's buffers.
struct HostStager;
struct HostSource {
  const uint64_t *rp;
  const void *col;
  cudaStream_t copy;
  void *labels_out = nullptr;  // host uint32 labels: each chunk is copied out on `copy`
                               // as soon as the final compression has finished it
  HostStager *stager = nullptr;  // when set: rows below 255 entries go as degree bytes
  bool sampled = false;  // sampled linking (tiled link rounds) instead of the tiled pass
  bool in_place = false;  // sampled: col of the Csr is the device address of the caller's
                          // page-locked ids, read in place; rp too unless offsets_copied
  bool offsets_copied = false;  // in place: the offsets cross in chunks (degree bytes)
  mutable uint64_t h2d_bytes = 0;  // bytes the pass copied to the device or read in place
};
void uf_components(const Csr &g, uint32_t *parent, const PartMap *pm,
                   const UfTuning &tu, cudaStream_t s, cudaMemPool_t pool,
                   Counters &c, const HostSource *hs = nullptr);
// The hook-schedule decisions on a stratified sample of (up to 8192) rows of a host
// CSR: the tiled pass suits it (< 50 % of the edges u < v leave their tile and
// < 10 % lie in rows above hub_degree); the link rounds of sampled linking stay
// in their tile (>= 75 % of the rows' link-round entries); few hub edges.
struct HostShares {
  bool tiles = false, link_tiles = false, few_hubs = true;
};
HostShares host_shares(const uint64_t *rp, const void *col, int idb, uint64_t n, uint64_t m,
                       uint32_t tile, uint32_t hub_degree, uint64_t max_samples = 8192);

// Write uint32 labels to an id_bytes-wide output array.
void widen_labels(const uint32_t *in, void *out, int out_bytes, uint64_t n,
                  cudaStream_t s, Counters &c);

// ---- scan / radix sort / component graph (sortcsr.cu) ----------------------
// Stable LSD radix sort of uint64 keys on bits [0, bits); returns the buffer
// (keys or tmp) that holds the result.
// (i, hist[i]) for every nonzero hist[i], i ascending, into pairs (2 words
// each, at most cap pairs); *d_count receives the number of nonzero entries.
void compact_histogram(const uint32_t *hist, uint64_t len, uint64_t *pairs, uint64_t cap,
                       uint32_t *d_count, cudaStream_t s, cudaMemPool_t pool, Counters &c);
// cnt[l] = vertices labelled l (n words), hist[k] = labels held by k vertices
// (n + 1 words); a label >= n is reported in *err.
void component_size_hist(const void *lab, int id_bytes, uint64_t n, uint32_t *cnt, uint32_t *hist,
                         int *err, cudaStream_t s, Counters &c);
// Adjacent-unique copy of n sorted keys into out; *d_count = number kept.
void unique_sorted_keys(const uint64_t *sorted, uint64_t n, uint64_t *out, uint32_t *d_count,
                        cudaStream_t s, cudaMemPool_t pool, Counters &c);
// Row offsets rp[0 .. count] of `count` rows from their degree bytes:
// rp[0] = base, rp[i + 1] = base + deg[0] + ... + deg[i] (the sum of one call
// must stay below 2^32).
void offsets_from_degrees(const uint8_t *deg, uint64_t count, uint64_t base, uint64_t *rp,
                          cudaStream_t s, cudaMemPool_t pool, Counters &c);
// The same with escapes: a degree byte of 255 stands for the exact degree of
// that row, found in esc (nesc (row, degree) pairs sorted by row; rows are
// absolute: first_row + i for entry i).
void offsets_from_degrees_esc(const uint8_t *deg, uint64_t count, uint64_t first_row, uint64_t base,
                              const uint2 *esc, uint32_t nesc, uint64_t *rp, cudaStream_t s,
                              cudaMemPool_t pool, Counters &c);
// The same from uint32 counts (the sum of one call must stay below 2^32).
void offsets_from_counts(const uint32_t *deg, uint64_t count, uint64_t base, uint64_t *rp,
                         cudaStream_t s, cudaMemPool_t pool, Counters &c);
uint64_t *radix_sort_u64(uint64_t *keys, uint64_t *tmp, uint64_t n, int bits,
                         cudaStream_t s, cudaMemPool_t pool, Counters &c);
// Stable ranks of n 8-bit digits: rank[i] = position of element i when the
// digits are sorted stably (ties in index order), inv[rank[i]] = i.
void stable_digit_ranks(const uint8_t *dig, uint64_t n, uint32_t *rank, uint32_t *inv,
                        cudaStream_t s, cudaMemPool_t pool, Counters &c);

// Result of contracting a graph along a vertex map.
struct Contracted {
  uint64_t n = 0, m = 0;
  DevBuf rp, col;   // CSR of the contracted graph (uint32 ids)
  DevBuf vid;       // per new vertex: original vertex id of its representative
  DevBuf newid;     // per old cluster id: new vertex id or kNone
};

// Build the quotient graph: for every edge (v,w) of g with
// cl[v] != cl[w] the undirected edge {cl[v], cl[w]}, deduplicated.  Cluster
// ids lie in [0, ncl).  New vertices are the clusters with at least one edge,
// numbered in increasing cluster-id order, so the order of cluster ids is
// kept.  vid_of_cluster maps a cluster id to the original vertex id carried
// over (nullptr = the cluster id itself).  With pm != nullptr only edges
// between different virtual ranks are kept (cut edges).
// Replaces CAGBuilder::PerformLocalContraction/BuildLocalContractionGraph
// (cag_builder.h:160-230, 577-667) and DynamicContraction's conflicting-edge
// routing and InsertAndClearEdges (dynamic_contraction.h:62-136, 251-290,
// 513-559): relabel, compact, sort, dedup, CSR rebuild.
void contract_graph(const Csr &g, const uint32_t *cl, uint64_t ncl,
                    const uint32_t *vid_of_cluster, const PartMap *pm,
                    Contracted &out, cudaStream_t s, cudaMemPool_t pool,
                    Counters &c, uint32_t *host_mailbox);

// ---- decomposition kernels (ldd.cu) ---------------------------------------
// Threshold table of the deviate sampler: dev >= k  iff  u < T[k-1], with
// T[k-1] = floor(2^64 exp(-beta k)), at most kGeoMax entries.
constexpr int kGeoMax = 4096;
int geo_table_build(double beta, std::vector<uint64_t> &t);
void geo_table_upload(double beta, uint64_t *d_table, int *len_out, cudaStream_t s);

// Row offsets of a caller's graph checked (rp[v] <= rp[v+1] <= m) into g.err.
void check_offsets(const Csr &g, cudaStream_t s, Counters &c);
// Bounds checks of a caller CSR (ids < n, offsets monotone and <= m; failures
// go to g.err) and, when col32 is given, a uint32 copy of its ids.  Used
// before kernels that assume a trusted uint32 graph.
void sanitize_ids(const Csr &g, uint32_t *col32, cudaStream_t s, Counters &c);

// Exponential-shift decomposition on g (exponential_contraction.h:439-628).
// key[i] = (dev_i << 32) | i; relaxes key[i] = min(key[i], key[j] + 2^32)
// over neighbours to the fixpoint.  cluster[i] = low 32 bits (centre index).
// Returns the number of rounds, or -1 if max_rounds was hit.
int ldd_decompose(const Csr &g, const uint32_t *vid, uint64_t seed, uint32_t level,
                  const uint64_t *d_geo, int geo_len, bool gated, uint32_t *cluster,
                  uint64_t *key, int max_rounds, cudaStream_t s, cudaMemPool_t pool,
                  Counters &c, volatile int *host_flag, int *dev_flag);

// Local contraction sweeps (local_contraction.h:157-300): uniform deviates in
// [0,99], then two Jacobi sweeps of the lexicographic minimum over N[v].
void local_sweeps(const Csr &g, const uint32_t *vid, uint64_t seed, uint32_t level,
                  uint32_t *cluster, cudaStream_t s, cudaMemPool_t pool, Counters &c);

// ---- propagation kernels (prop.cu) -----------------------------------------
// Min-label propagation rounds (propagation.h:72-149) on lab (in place).
// Round loops return the number of rounds, -1 when max_rounds ran out, and
// kRoundsBadInput when g.err is set (the caller's ids not checked yet: the
// first round checks them) and an id was out of range; *g.err holds the code.
constexpr int kRoundsBadInput = -2;
int labels_propagate(const Csr &g, uint32_t *lab, int max_rounds, cudaStream_t s,
                     cudaMemPool_t pool, Counters &c, volatile int *host_flag, int *dev_flag);
// Shortcut propagation rounds (shortcut_propagation.h:124-376).
int shortcut_propagate(const Csr &g, uint32_t *lab, uint32_t hitters, int max_rounds,
                       cudaStream_t s, cudaMemPool_t pool, Counters &c,
                       volatile int *host_flag, int *dev_flag);

// out[i] = lab_next[newid[cl[i]]] if newid[cl[i]] != kNone else rep[cl[i]]
// (label composition, replaces DynamicContraction::UndoContraction,
// dynamic_contraction.h:568-658).
void compose_labels(const uint32_t *cl, const uint32_t *newid, const uint32_t *lab_next,
                    const uint32_t *rep, uint32_t *out, uint64_t n, cudaStream_t s,
                    Counters &c);
// lab[v] <- minimum vertex id among all u with lab[u] == lab[v]; lab values are
// vertex ids in [0, n).  scratch: n uint32.
void canonicalize(uint32_t *lab, uint32_t *scratch, uint64_t n, cudaStream_t s, Counters &c);
// Count v with lab[v] == v (components, canonical labels).
void count_roots(const uint32_t *lab, uint64_t n, unsigned long long *d_count,
                 cudaStream_t s, Counters &c);
// Gather: out[i] = src[idx[i]]
void gather_u32(const uint32_t *src, const uint32_t *idx, uint32_t *out, uint64_t n,
                cudaStream_t s, Counters &c);
void iota_u32(uint32_t *out, uint64_t n, cudaStream_t s, Counters &c);

}  // namespace ccg

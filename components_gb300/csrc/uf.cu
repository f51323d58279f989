// uf.cu - hook-and-compress connected components (lock-free union-find).
//
// Replaces the sequential BFS of the reference's base case and local pass:
//   Utility::BFS                       lib/components/utils.h:37-58
//   FindLocalComponents                exponential_contraction.h:391-411
//   AllReduce::FindComponentsOnRoot    all_reduce.h:110-139
// The BFS labels every vertex with the first vertex of its component in
// ascending order, i.e. the minimum id.  Here every link points from the larger
// root to the smaller one (parent[x] <= x always), so the surviving root of a
// component is its minimum vertex id and the result is the same label.
//
// Layout: one uint32 parent word per vertex; the CSR is read once, in vertex
// order.  Low-degree vertices are handled one per thread; vertices above the
// hub degree are queued and handled one per warp so that a hub does not stall
// its warp (RHG hubs reach degrees in the tens of thousands).
//
// The kernels read the caller's CSR directly, so every offset and id is
// checked: a bad one is recorded in the error word and skipped.
#include <algorithm>
#include <vector>

#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "hostpool.h"
#include "kernels.h"

namespace ccg {
namespace {

// Root of v with path halving.  parent[] only ever decreases along a path,
// so a stale read still names an ancestor and writes only shorten paths.  The
// walk's loads go through L1: a cached entry may be stale, but the walk then
// ends at a node that was a root when cached; unions built on it stay exact
// because the CAS that links checks the root on the L2 copy and hands back the
// current parent when it fails.  Hot entries (the root of a big component, a
// hub) are then served by L1 instead of all reading one L2 line.
__device__ __forceinline__ uint32_t uf_find_l1(uint32_t *p, uint32_t v) {
  uint32_t cur = p[v];
  if (cur == v) return v;
  uint32_t prev = v;
  uint32_t next;
  while (cur > (next = p[cur])) {
    st_cg(p + prev, next);
    prev = cur;
    cur = next;
  }
  return cur;
}

// Link the trees of a and b: the larger root is CAS'ed under the smaller one.
// The finds read through L1 (uf_find_l1); the CAS decides.
__device__ __forceinline__ void uf_union(uint32_t *p, uint32_t a, uint32_t b) {
  uint32_t ra = uf_find_l1(p, a), rb = uf_find_l1(p, b);
  while (ra != rb) {
    if (ra < rb) {
      uint32_t t = ra;
      ra = rb;
      rb = t;
    }
    uint32_t old = atomicCAS(p + ra, ra, rb);
    if (old == ra) return;
    ra = uf_find_l1(p, old);
    rb = uf_find_l1(p, rb);
  }
}

// Lower bound of v's virtual rank.
__device__ __forceinline__ uint32_t part_lo(const PartMap &pm, uint32_t v) {
  uint32_t r = pm.part(v);
  return r < pm.rm ? r * (pm.q + 1) : pm.big + (r - pm.rm) * pm.q;
}

struct Row {
  uint64_t b, e;
};
// Offsets of row v, checked against m.
__device__ __forceinline__ bool load_row(const uint64_t *__restrict__ rp, uint64_t v, uint64_t m,
                                         int *err, Row &r) {
  r.b = __ldg(rp + v);
  r.e = __ldg(rp + v + 1);
  if (r.e < r.b || r.e > m) {
    set_err(err, kErrBadOffsets);
    return false;
  }
  return true;
}

// parent[v] = first neighbour if it is smaller (and in v's rank), else v.
template <class T, bool PART>
__global__ void k_init(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                       const T *__restrict__ col, uint32_t *__restrict__ p, PartMap pm, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    Row r;
    uint32_t par = (uint32_t)v;
    if (load_row(rp, v, m, err, r) && r.b < r.e) {
      uint64_t u = (uint64_t)__ldg(col + r.b);
      if (u >= n) set_err(err, kErrBadId);  // k_hook checks the other entries
      bool ok = u < v;
      if (PART && ok) ok = (uint32_t)u >= part_lo(pm, (uint32_t)v);
      if (ok) par = (uint32_t)u;
    }
    p[v] = par;
  }
}

// Where the hook kernel sends a row above hub_degree: a plain list of rows
// (one warp per row later; the fixed-scratch solve) or warp-sized pieces.
struct RowSink {
  uint32_t *hubs;
  uint64_t cap;
  unsigned int *count;
  __device__ __forceinline__ void put(uint32_t v, uint64_t, int *err) const {
    const uint32_t slot = atomicAdd(count, 1u);
    if (slot < cap) hubs[slot] = v;
    else set_err(err, kErrOverflow);
  }
};

template <class T, bool PART, class Sink>
__global__ void k_hook(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                       const T *__restrict__ col, uint32_t *p, PartMap pm, uint32_t hub_degree,
                       Sink sink, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    Row r;
    if (!load_row(rp, v, m, err, r)) continue;
    if (r.e - r.b > hub_degree) {
      sink.put((uint32_t)v, r.e - r.b, err);
      continue;
    }
    uint32_t lo = PART ? part_lo(pm, (uint32_t)v) : 0u;
    // the first neighbour was linked by k_init when it qualified
    for (uint64_t k = r.b + 1; k < r.e; ++k) {
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        continue;
      }
      if (u < v && (!PART || (uint32_t)u >= lo)) uf_union(p, (uint32_t)v, (uint32_t)u);
    }
  }
}

// One warp per hub vertex; lanes stride over its adjacency.
template <class T, bool PART>
__global__ void k_hook_hubs(uint64_t n, const uint64_t *__restrict__ rp,
                            const T *__restrict__ col, uint32_t *p, PartMap pm,
                            const uint32_t *__restrict__ hubs, uint64_t hub_cap,
                            const unsigned int *__restrict__ nhubs, int *err) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t nh = *nhubs;
  if (nh > hub_cap) nh = hub_cap;
  for (uint64_t h = warp; h < nh; h += nwarps) {
    uint32_t v = hubs[h];
    uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);  // checked by k_hook
    uint32_t lo = PART ? part_lo(pm, v) : 0u;
    for (uint64_t k = b + 1 + lane; k < e; k += 32) {
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        continue;
      }
      if (u < v && (!PART || (uint32_t)u >= lo)) uf_union(p, v, (uint32_t)u);
    }
  }
}

// Full compression: parent[v] <- root.  Runs after every link is made.  Only
// v's own entry is written: a halving store into p[x] could land after x's own
// thread wrote its root (and leave x at an inner node), and writing the root
// along the whole path was measured slower (store traffic on shared paths).
// The walk reads through L1: roots do not change any more, and a stale inner
// entry still names an ancestor, so a cached read is always a valid step; the
// cache keeps a giant component's root entry from becoming one hot L2 line
// that every vertex reads.
// Each thread walks kCompressWays vertices' chains side by side (v, v + stride,
// ..., coalesced across the warp), so that many dependent loads are in flight.
constexpr int kCompressWays = 2;  // measured: 2 beats 1 and 4 on the grid and the hyperbolic graph
__global__ void k_compress(uint64_t n, uint32_t *p, uint64_t v_begin = 0) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t a = v_begin + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; a < n;
       a += kCompressWays * stride) {
    uint32_t r0[kCompressWays], x[kCompressWays];
    bool done[kCompressWays];
#pragma unroll
    for (int k = 0; k < kCompressWays; ++k) {
      const uint64_t v = a + k * stride;
      r0[k] = v < n ? p[v] : (uint32_t)v;
      x[k] = r0[k];
      done[k] = v >= n || r0[k] == (uint32_t)v;
    }
    bool all = true;
#pragma unroll
    for (int k = 0; k < kCompressWays; ++k) all &= done[k];
    while (!all) {
      uint32_t nx[kCompressWays];
#pragma unroll
      for (int k = 0; k < kCompressWays; ++k) nx[k] = done[k] ? x[k] : p[x[k]];
      all = true;
#pragma unroll
      for (int k = 0; k < kCompressWays; ++k) {
        if (!done[k]) {
          if (nx[k] == x[k]) done[k] = true;
          else x[k] = nx[k];
        }
        all &= done[k];
      }
    }
#pragma unroll
    for (int k = 0; k < kCompressWays; ++k) {
      const uint64_t v = a + k * stride;
      if (v < n && x[k] != r0[k]) p[v] = x[k];  // most vertices already point at their root
    }
  }
}

// Hub rows are split into pieces of kPiece edges, one warp per piece, so that
// one row of a million edges is spread over hundreds of warps.
constexpr uint32_t kPiece = 2048;
struct HubList {
  uint2 *items;  // (row, piece index)
  uint64_t cap;
  unsigned int *count;
};
// Pieces needed for hub rows of a graph with m edges and rows above hub_degree.
inline uint64_t hub_list_cap(uint64_t m, uint32_t hub_degree) {
  return m / ((uint64_t)hub_degree + 1) + m / kPiece + 2;
}
__device__ __forceinline__ void queue_hub(const HubList &hl, uint32_t v, uint64_t len, int *err) {
  const uint32_t np = (uint32_t)((len + kPiece - 1) / kPiece);
  if (np == 0) return;
  const unsigned int slot = atomicAdd(hl.count, np);
  if ((uint64_t)slot + np > hl.cap) {
    set_err(err, kErrOverflow);
    return;
  }
  for (uint32_t q = 0; q < np; ++q) hl.items[slot + q] = make_uint2(v, q);
}
struct PieceSink {
  HubList hl;
  __device__ __forceinline__ void put(uint32_t v, uint64_t len, int *err) const {
    queue_hub(hl, v, len, err);
  }
};

// ---- sampled linking (Afforest: Sutton, Ben-Nun, Barak, IPDPS 2018) ------------
// Link every vertex to kAffRounds of its neighbours, compress, find
// the most frequent root L on a sample, then only vertices outside L's tree
// process their remaining edges.  An edge skipped by an endpoint inside L is
// either processed from its other endpoint or joins two vertices that are
// already connected, so the components are exact.  On graphs with a giant
// component most edges are never touched; without one it costs two light
// passes.
constexpr uint32_t kAffRounds = 2;

// Entry of row v (d entries) that link round r uses (r < min(d, kAffRounds)).
// One rank (ALT false): the row's first entries.  On sorted rows these are the
// smallest neighbour ids, which on hyperbolic graphs are often hubs: the link
// rounds then already join the giant component (entries spread through the
// row were measured to leave it in pieces).  Alternating by row parity (odd
// rows their last entries) made that pass 21 % slower: a larger neighbour
// cannot take the one-CAS hook and goes through the union queue.
// Virtual ranks (ALT true): even rows their first entries, odd rows their
// last.  With ranks the link rounds skip the entries that leave the rank, and
// with the first entries the tile-crossing link edges that remain pile onto
// a few vertices per rank: their global unions took 1.0-1.25 ms on the
// 2^26-vertex hyperbolic graph with 16 ranks, against 0.26 ms alternating.
// Which entries the rounds take changes no component, only the work.
template <bool ALT>
__host__ __device__ __forceinline__ uint64_t link_pos(uint64_t v, uint64_t d, uint32_t r) {
  return (ALT && (v & 1)) ? d - 1 - r : (uint64_t)r;
}
template <bool ALT>
__host__ __device__ __forceinline__ bool is_link_pos(uint64_t v, uint64_t d, uint64_t j) {
  for (uint32_t r = 0; r < kAffRounds && r < d; ++r)
    if (link_pos<ALT>(v, d, r) == j) return true;
  return false;
}

template <class T, bool PART>
__global__ void k_aff_link(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                           const T *__restrict__ col, uint32_t *p, PartMap pm, uint32_t r, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    Row row;
    if (!load_row(rp, v, m, err, row) || row.e - row.b <= r) continue;
    const uint64_t u = (uint64_t)__ldg(col + row.b + link_pos<PART>(v, row.e - row.b, r));
    if (u >= n) {
      set_err(err, kErrBadId);
      continue;
    }
    uint32_t lo = 0, hi = 0xffffffffu;
    if (PART) pm.bounds((uint32_t)v, lo, hi);
    if ((uint32_t)u >= lo && (uint32_t)u < hi) uf_union(p, (uint32_t)v, (uint32_t)u);
  }
}

// `per` sampled roots for each of `nparts` partitions (nparts = 1: the whole
// graph): a partition's most frequent root is its giant local component.
__global__ void k_aff_sample(uint64_t n, const uint32_t *p, PartMap pm, uint32_t nparts,
                             uint32_t per, uint64_t salt, uint32_t *__restrict__ out) {
  const uint32_t samples = nparts * per;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < samples; i += gridDim.x * blockDim.x) {
    const uint64_t h = mix64(salt + i);
    uint64_t lo = 0, len = n;
    if (nparts > 1) {
      const uint32_t q = i / per;
      lo = q < pm.rm ? (uint64_t)q * (pm.q + 1) : (uint64_t)pm.big + (uint64_t)(q - pm.rm) * pm.q;
      len = q < pm.rm ? pm.q + 1 : pm.q;
    }
    uint32_t r = (uint32_t)(lo + h % len), nx;
    while ((nx = ld_cg(p + r)) != r) r = nx;
    out[i] = r;
  }
}

// Most frequent value among the `per` (<= kModeBlock) samples of block q
// (ties: the smallest value): a bitonic sort in shared memory, each run's
// length by a binary search for its end, then a block-wide maximum of
// (length, ~value).
constexpr int kModeBlock = 1024;
__global__ void __launch_bounds__(kModeBlock) k_aff_mode(const uint32_t *__restrict__ smp, uint32_t per,
                                                        uint32_t *__restrict__ Ls) {
  __shared__ uint32_t a[kModeBlock];
  __shared__ unsigned long long best[kModeBlock / 32];
  const uint32_t i = threadIdx.x;
  a[i] = i < per ? smp[(uint64_t)blockIdx.x * per + i] : 0xffffffffu;
  __syncthreads();
  for (uint32_t k = 2; k <= kModeBlock; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      const uint32_t ixj = i ^ j;
      if (ixj > i) {
        const uint32_t x = a[i], y = a[ixj];
        if ((i & k) == 0 ? x > y : x < y) {
          a[i] = y;
          a[ixj] = x;
        }
      }
      __syncthreads();
    }
  }
  unsigned long long key = 0;
  if (i < per && (i == 0 || a[i] != a[i - 1])) {
    uint32_t lo = i, hi = per;  // first index past the run of a[i]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) / 2;
      if (a[mid] == a[i]) lo = mid;
      else hi = mid;
    }
    key = ((unsigned long long)(lo + 1 - i) << 32) | (0xffffffffu - a[i]);
  }
  for (int o = 16; o; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, key, o);
    key = y > key ? y : key;
  }
  if ((i & 31) == 0) best[i >> 5] = key;
  __syncthreads();
  if (i < 32) {
    key = best[i];
    for (int o = 16; o; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, key, o);
      key = y > key ? y : key;
    }
    if (i == 0) Ls[blockIdx.x] = key ? 0xffffffffu - (uint32_t)key : kNone;
  }
}

template <class T, bool PART>
__global__ void k_aff_rest(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                           const T *__restrict__ col, uint32_t *p, PartMap pm,
                           const uint32_t *__restrict__ Ls, uint32_t nparts,
                           uint32_t hub_degree, HubList hl, int *err,
                           unsigned long long *__restrict__ edges_read) {
  uint32_t work = 0, rows = 0;  // neighbour ids and offset pairs this thread reads
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    // the root first: rows inside the giant component never read their offsets.
    // The parents were compressed before this pass, so p[v] == L settles most
    // rows with one coalesced load (and no read of L's own, hot, entry).
    const uint32_t L = nparts > 1 ? Ls[pm.part((uint32_t)v)] : Ls[0];
    if (ld_cg(p + v) == L || uf_find_l1(p, (uint32_t)v) == L) continue;
    ++rows;
    Row row;
    if (!load_row(rp, v, m, err, row) || row.e - row.b <= kAffRounds) continue;
    if (row.e - row.b > hub_degree) {
      queue_hub(hl, (uint32_t)v, row.e - row.b, err);
      continue;
    }
    work += (uint32_t)(row.e - row.b - kAffRounds);
    uint32_t lo = 0, hi = 0xffffffffu;  // v's rank
    if (PART) pm.bounds((uint32_t)v, lo, hi);
    for (uint64_t k = row.b; k < row.e; ++k) {
      if (is_link_pos<PART>(v, row.e - row.b, k - row.b)) continue;  // linked already
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        continue;
      }
      if ((uint32_t)u >= lo && (uint32_t)u < hi) uf_union(p, (uint32_t)v, (uint32_t)u);
    }
  }
  if (edges_read) {  // every thread of the warp reaches this point
    work = __reduce_add_sync(0xffffffffu, work);
    rows = __reduce_add_sync(0xffffffffu, rows);
    if ((threadIdx.x & 31) == 0) {
      if (work) atomicAdd(edges_read, (unsigned long long)work);
      if (rows) atomicAdd(edges_read + 1, (unsigned long long)rows);
    }
  }
}

// One warp per hub piece: edges [y*kPiece, (y+1)*kPiece) of row x.  LESS:
// only edges to smaller ids (hook/tile passes, each undirected edge once);
// otherwise every edge but the row's link-round entries (the sampled pass skips
// rows inside the giant component, so an edge may be seen from one end only).
template <class T, bool PART, bool LESS>
__global__ void k_hub_pieces(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                             const T *__restrict__ col, uint32_t *p, PartMap pm, HubList hl,
                             int *err) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t cnt = *hl.count;
  if (cnt > hl.cap) cnt = hl.cap;  // an overflow was recorded; unwritten items are skipped below
  for (uint64_t h = warp; h < cnt; h += nwarps) {
    const uint2 it = hl.items[h];
    const uint32_t v = it.x;
    if (v >= n) continue;
    const uint64_t rb = __ldg(rp + v), re = __ldg(rp + v + 1);
    if (re < rb || re > m) continue;  // recorded by the pass that queued the row
    const uint64_t b = rb + (uint64_t)it.y * kPiece;
    const uint64_t e = min(re, b + kPiece);
    uint32_t lo = 0, hi = 0xffffffffu;  // v's rank
    if (PART) pm.bounds(v, lo, hi);
    for (uint64_t k = b + lane; k < e; k += 32) {
      const uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        continue;
      }
      if (LESS) {
        if (u < v && (uint32_t)u >= lo) uf_union(p, v, (uint32_t)u);
      } else if (!is_link_pos<PART>(v, re - rb, k - rb)) {  // the link rounds took those
        if ((uint32_t)u >= lo && (uint32_t)u < hi) uf_union(p, v, (uint32_t)u);
      }
    }
  }
}

__global__ void k_iota_parent(uint64_t n, uint32_t *p) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    p[v] = (uint32_t)v;
}

// ---- tiled pass ---------------------------------------------------------------
// One CTA per tile of TILE consecutive vertices: the edges inside the tile are
// united on a parent array in shared memory (chains resolve at shared-memory
// latency instead of L2 latency), every vertex then stores the global id of
// its tile-local root, and only the edges that leave the tile go to a global
// list.  This is the reference's partition-local pass with the CTA as the
// rank (FindLocalComponents, exponential_contraction.h:391-411).
// Shared-memory parent entries are 16 bits wide in the hook pass and 32 bits
// in link mode (TileParent below).
__device__ __forceinline__ uint64_t shfl64(uint64_t x, int src) {
  const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)x, src);
  const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(x >> 32), src);
  return ((uint64_t)hi << 32) | lo;
}

// The tile kernel.  Warps take 32 consecutive rows at a time and walk the
// rows' edges as one flattened, coalesced stream (lane k reads edge k of the
// 32 rows' concatenated adjacency; its row comes from a binary search over
// the warp's degree prefix sums).  Edges inside the tile go to a per-warp
// queue in shared memory and are united 32 at a time, so every lane of a
// union step has work.  Edges leaving the tile are staged in shared memory
// (one global atomic per tile) and written out with their near end replaced
// by its tile-local root; when the stage is full they go straight to the
// global list with the raw near end.  Every vertex finally stores the global
// id of its tile-local root.
constexpr uint32_t kUnionQueue = 64;  // per warp: < 32 pending + up to 32 new
constexpr uint32_t kTileMax = 65536;  // queue entries pack two 16-bit tile indices
// CTAs per SM of the cut union: the tiled pass's tile-crossing edges have
// distinct endpoints and more threads in flight hide their latency (8192^2
// grid: 0.270 / 0.246 / 0.224 ms at 16 / 32 / 64); the link rounds' crossing
// edges pile onto a few hub roots, where more concurrent CASes fail and retry
// (2^26 hyperbolic graph: 0.29 / 0.54 / 0.41 ms).
constexpr unsigned kCutCtasTiled = 64, kCutCtasLink = 16;
constexpr uint32_t kLinkGroups = 1;   // link mode: 32-row blocks per warp step (1 measured best of 1, 2, 4)
// Parent entries of a tile in shared memory: 16 bits in the hook pass (twice
// the vertices for the same shared memory: fewer tile-crossing edges on
// grids), 32 bits in link mode with half the vertices.  Link mode hooks all
// 32 rows of a warp at once, and a 16-bit CAS shares its 32-bit word with the
// neighbouring row's entry: on the 2^26-vertex hyperbolic graph the link pass
// took 1.10 ms on 16-bit entries (32768-vertex tiles) and 1.02 ms on 32-bit
// entries (16384-vertex tiles), the 16-rank link pass 1.37 and 1.18 ms.
template <int LINK>
using TileParent = std::conditional_t<(LINK > 0), uint32_t, uint16_t>;

template <class PT>
size_t tile_smem_bytes(uint32_t tile, uint32_t threads, uint32_t stage) {
  return (size_t)tile * sizeof(PT) + (size_t)(threads / 32) * kUnionQueue * 4 + (size_t)stage * 8;
}

// LINK = 0: every edge to a smaller id (the tiled hook pass; rows above
// hub_degree are queued as hub pieces).  LINK = k > 0: the k link-round entries
// of every row (link_pos) in either direction (the link rounds of sampled
// linking, which stay inside their tile on geometric and angularly ordered
// graphs).
template <class T, bool PART, class PT, int LINK>
__global__ void __launch_bounds__(1024, 2)
    k_tile3(uint64_t n, uint64_t m, uint64_t v_begin, uint64_t v_end,
            const uint64_t *__restrict__ rp, const T *__restrict__ col,
            uint32_t *__restrict__ p, PartMap pm, uint32_t tile, uint32_t stage_cap,
            uint32_t hub_degree, HubList hl, uint2 *__restrict__ cut, uint64_t cut_cap,
            unsigned long long *__restrict__ ncut, int *err) {
  extern __shared__ __align__(16) unsigned char tile_smem[];
  // layout: cut stage (8-byte entries), union queues, tile parents
  uint2 *cstage = reinterpret_cast<uint2 *>(tile_smem);
  uint32_t *queues = reinterpret_cast<uint32_t *>(cstage + stage_cap);
  volatile PT *s = reinterpret_cast<volatile PT *>(queues + (blockDim.x / 32) * kUnionQueue);
  __shared__ unsigned int ccount;
  __shared__ unsigned long long cbase;
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  uint32_t *q = queues + wid * kUnionQueue;
  for (uint64_t t0 = v_begin + (uint64_t)blockIdx.x * tile; t0 < v_end;
       t0 += (uint64_t)gridDim.x * tile) {
    const uint32_t len = (uint32_t)min((uint64_t)tile, v_end - t0);
    const uint32_t tt = (uint32_t)t0;
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) s[i] = (PT)i;
    if (threadIdx.x == 0) ccount = 0;
    __syncthreads();
    uint32_t qn = 0;  // warp-uniform queue fill
    // One edge (v, uu) per lane, all lanes together: an in-tile edge to a
    // smaller id goes to the warp's union queue (32 queued entries make a
    // union step), an edge to an earlier tile to the cut stage.
    // hook: the lane's row may link itself under its first in-tile smaller
    // neighbour with one CAS (no finds) while it is still a root; a link
    // under a non-root keeps parents smaller than children, so the forest
    // stays acyclic.  Only the row-per-lane loops hook.
    bool hooked = false;
    auto edge = [&](bool valid, uint64_t uu, uint32_t vi, uint32_t lov, uint32_t hiv,
                    bool may_hook) {
      const uint32_t vv = tt + vi;
      bool uni = false, emit = false;
      uint32_t u = 0;
      if (valid) {
        if (uu >= n) {
          set_err(err, kErrBadId);
        } else if (LINK) {
          if ((uint32_t)uu != vv && (!PART || ((uint32_t)uu >= lov && (uint32_t)uu < hiv))) {
            u = (uint32_t)uu;
            if (u >= tt && u - tt < len) {
              if (may_hook && !hooked && u < vv) {  // the hook needs a smaller parent
                hooked = true;
                uni = smem_cas(const_cast<PT *>(s + vi), vi, u - tt) != vi;
              } else {
                uni = true;
              }
            } else {
              emit = true;  // a cut edge in either direction
            }
          }
        } else if ((uint32_t)uu < vv && (!PART || (uint32_t)uu >= lov)) {
          u = (uint32_t)uu;  // each undirected edge once, from its larger end
          if (u < tt) {
            emit = true;
          } else if (may_hook && !hooked) {
            hooked = true;
            uni = smem_cas(const_cast<PT *>(s + vi), vi, u - tt) != vi;  // hooked, or queue
          } else {
            uni = true;
          }
        }
      }
      const unsigned um = __ballot_sync(0xffffffffu, uni);
      if (uni) q[qn + __popc(um & lt)] = vi | ((u - tt) << 16);
      qn += __popc(um);
      if (qn >= 32) {  // a full union step: the newest 32 entries
        __syncwarp();
        const uint32_t w = q[qn - 32 + lane];
        smem_union<true>(s, w & 0xffffu, w >> 16);
        qn -= 32;
        __syncwarp();
      }
      const unsigned em = __ballot_sync(0xffffffffu, emit);
      if (em) {
        unsigned int base = 0;
        if (lane == (unsigned)(__ffs(em) - 1)) base = atomicAdd(&ccount, (unsigned)__popc(em));
        base = __shfl_sync(0xffffffffu, base, __ffs(em) - 1);
        const unsigned int slot = base + __popc(em & lt);
        const bool over = emit && slot >= stage_cap;
        if (emit && !over) cstage[slot] = make_uint2(vi, u);  // near end as a tile index for now
        const unsigned om = __ballot_sync(0xffffffffu, over);
        if (om) {
          unsigned long long gb = 0;
          if (lane == (unsigned)(__ffs(om) - 1)) gb = atomicAdd(ncut, (unsigned long long)__popc(om));
          gb = __shfl_sync(0xffffffffu, gb, __ffs(om) - 1);
          if (over) {
            const unsigned long long gs = gb + __popc(om & lt);
            if (gs < cut_cap) cut[gs] = make_uint2(vv, u);
            else set_err(err, kErrOverflow);
          }
        }
      }
    };
    if constexpr (LINK > 0) {
      // Link mode reads at most LINK entries per row, so every warp takes
      // kLinkGroups blocks of 32 rows at once (lane = row) and issues all of
      // their offset loads, then all of their id loads, before any
      // shared-memory work: the pass is bound by the latency of these two
      // dependent loads, not by issue.
      constexpr uint32_t R = kLinkGroups;
      for (uint32_t g0 = wid * 32 * R; g0 < len; g0 += nw * 32 * R) {
        uint64_t rb[R], re[R];
#pragma unroll
        for (uint32_t r = 0; r < R; ++r) {
          const uint32_t i = g0 + 32 * r + lane;
          rb[r] = re[r] = 0;
          if (i < len) {
            rb[r] = __ldg(rp + t0 + i);
            re[r] = __ldg(rp + t0 + i + 1);
          }
        }
        uint32_t deg[R];
#pragma unroll
        for (uint32_t r = 0; r < R; ++r) {
          deg[r] = 0;
          if (re[r] < rb[r] || re[r] > m) set_err(err, kErrBadOffsets);
          else deg[r] = (uint32_t)min(re[r] - rb[r], (uint64_t)LINK);
        }
        T id[R][LINK];
#pragma unroll
        for (uint32_t r = 0; r < R; ++r)
#pragma unroll
          for (uint32_t j = 0; j < (uint32_t)LINK; ++j)
            id[r][j] = j < deg[r] ? __ldg(col + rb[r] + link_pos<PART>(t0 + g0 + 32 * r + lane, re[r] - rb[r], j)) : (T)0;
#pragma unroll
        for (uint32_t r = 0; r < R; ++r) {
          const uint32_t i = g0 + 32 * r + lane;
          uint32_t lo = 0, hi = 0xffffffffu;  // v's rank (PART)
          if (PART && i < len) pm.bounds(tt + i, lo, hi);
          const uint32_t maxdeg = __reduce_max_sync(0xffffffffu, deg[r]);
          hooked = false;
#pragma unroll
          for (uint32_t j = 0; j < (uint32_t)LINK; ++j)
            if (j < maxdeg) edge(j < deg[r], (uint64_t)id[r][j], i, lo, hi, true);
        }
      }
    } else {
      for (uint32_t g0 = wid * 32; g0 < len; g0 += nw * 32) {
        const uint32_t i = g0 + lane;
        uint64_t rb = 0;  // row start
        uint32_t deg = 0, lo = 0, hi = 0xffffffffu;  // lo, hi: v's rank (PART)
        if (i < len) {
          const uint64_t v = t0 + i;
          rb = __ldg(rp + v);
          const uint64_t re = __ldg(rp + v + 1);
          if (re < rb || re > m) {
            set_err(err, kErrBadOffsets);
          } else if (re - rb > hub_degree) {
            queue_hub(hl, (uint32_t)v, re - rb, err);
          } else {
            deg = (uint32_t)(re - rb);
            if (PART) pm.bounds((uint32_t)v, lo, hi);
          }
        }
        hooked = false;
        const uint32_t maxdeg = __reduce_max_sync(0xffffffffu, deg);
        const uint32_t total = __reduce_add_sync(0xffffffffu, deg);
        if (maxdeg <= 2 * ((total + 31) / 32) + 1) {
          // even degrees: lane = row, maxdeg steps, the ids of 32 neighbouring
          // rows are adjacent in memory.  A step where no lane holds an edge to
          // a smaller id (or a bad id) has nothing to unite or emit and skips
          // the edge logic: on sorted rows the later entries are the larger
          // neighbours.
          for (uint32_t j = 0; j < maxdeg; ++j) {
            const bool valid = j < deg;
            const uint64_t uu = valid ? (uint64_t)__ldg(col + rb + j) : 0ull;
            if (__any_sync(0xffffffffu, valid && (uu >= n || (uint32_t)uu < tt + i)))
              edge(valid, uu, i, lo, hi, true);
          }
        } else {
          // skewed degrees: the 32 rows' edges as one flattened stream, lane k
          // reads entry k; its row is the last lane whose prefix sum is <= k
          uint32_t inc = deg;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if ((int)lane >= o) inc += t;
          }
          const uint32_t off = inc - deg;
          for (uint32_t f0 = 0; f0 < total; f0 += 32) {
            const uint32_t f = f0 + lane;
            int r = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1) {
              const uint32_t o = __shfl_sync(0xffffffffu, off, r + step);
              if (o <= f) r += step;
            }
            const uint32_t ro = __shfl_sync(0xffffffffu, off, r);
            const uint64_t rbr = shfl64(rb, r);
            const uint32_t lor = PART ? __shfl_sync(0xffffffffu, lo, r) : 0u;
            const bool valid = f < total;
            edge(valid, valid ? (uint64_t)__ldg(col + rbr + (f - ro)) : 0ull, g0 + (uint32_t)r, lor,
                 0xffffffffu, false);
          }
        }
      }
    }
    __syncwarp();
    if (lane < qn) {  // the queue's remainder
      const uint32_t w = q[lane];
      smem_union<true>(s, w & 0xffffu, w >> 16);
    }
    __syncthreads();
    // every vertex stores the global id of its tile-local root
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) p[t0 + i] = tt + smem_find(s, i);
    const unsigned int nc = min(ccount, stage_cap);
    if (LINK) {
      // Link rounds: many rows of a tile link to the same far vertex (a hub),
      // and after the near end becomes its tile-local root most staged edges
      // repeat.  Duplicates are dropped through a hash set in the (now idle)
      // union-queue memory; a key that finds no free slot in a few probes is
      // kept, so the set only ever removes true repeats.
      unsigned long long *set = reinterpret_cast<unsigned long long *>(queues);
      const uint32_t slots = nw * kUnionQueue / 2;
      for (uint32_t k = threadIdx.x; k < slots; k += blockDim.x) set[k] = ~0ull;
      __syncthreads();  // every thread has read ccount into nc
      if (threadIdx.x == 0) ccount = 0;  // reused: kept edges
      __syncthreads();
      for (uint32_t k = threadIdx.x; k < nc; k += blockDim.x) {
        uint2 c = cstage[k];
        c.x = tt + smem_find(s, c.x);
        const unsigned long long key = ((unsigned long long)c.x << 32) | c.y;
        uint32_t h = (uint32_t)(mix64(key) % slots);
        bool keep = true;
        for (int probe = 0; probe < 8; ++probe) {
          const unsigned long long old = atomicCAS(set + h, ~0ull, key);
          if (old == ~0ull) break;
          if (old == key) {
            keep = false;
            break;
          }
          h = h + 1 == slots ? 0 : h + 1;
        }
        if (keep) atomicAdd(&ccount, 1u);
        else c.y = kNone;  // ids are < n <= 2^32 - 2, so kNone marks a dropped edge
        cstage[k] = c;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        cbase = ccount ? atomicAdd(ncut, (unsigned long long)ccount) : 0ull;
        ccount = 0;  // reused: fill position
      }
      __syncthreads();
      for (uint32_t k = threadIdx.x; k < nc; k += blockDim.x) {
        const uint2 c = cstage[k];
        if (c.y == kNone) continue;
        const unsigned long long g = cbase + atomicAdd(&ccount, 1u);
        if (g < cut_cap) cut[g] = c;
        else set_err(err, kErrOverflow);
      }
    } else {
      if (threadIdx.x == 0) cbase = nc ? atomicAdd(ncut, (unsigned long long)nc) : 0ull;
      __syncthreads();
      for (uint32_t k = threadIdx.x; k < nc; k += blockDim.x) {
        const uint2 c = cstage[k];
        const unsigned long long g = cbase + k;
        if (g < cut_cap) cut[g] = make_uint2(tt + smem_find(s, c.x), c.y);
        else set_err(err, kErrOverflow);
      }
    }
    __syncthreads();
  }
}

// Edges between tiles, on the global parent array of tile-local roots.  After
// each union an endpoint whose parent is not yet the common root it saw is
// pointed at it (an ancestor of both; an endpoint other than that root already
// has a parent, so no CAS can target it).  The store is skipped when the entry
// already holds the root: many cut edges share a few endpoints (a tile root, a
// hub), and repeated stores into those hot entries serialise in L2.
// Entries [*from, *ncut) of the list (from null: all of it).
__global__ void k_cut_union(const uint2 *__restrict__ cut, const unsigned long long *__restrict__ ncut,
                            uint64_t cut_cap, uint32_t *p,
                            const unsigned long long *__restrict__ from = nullptr) {
  uint64_t cnt = *ncut;
  if (cnt > cut_cap) cnt = cut_cap;
  const uint64_t first = from ? *from : 0;
  for (uint64_t i = first + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint2 e = cut[i];
    uint32_t ra = uf_find_l1(p, e.x), rb = uf_find_l1(p, e.y);
    while (ra != rb) {
      if (ra < rb) {
        const uint32_t t = ra;
        ra = rb;
        rb = t;
      }
      const uint32_t old = atomicCAS(p + ra, ra, rb);
      if (old == ra) {
        ra = rb;
        break;
      }
      ra = uf_find_l1(p, old);
      rb = uf_find_l1(p, rb);
    }
    if (e.x != ra && ld_cg(p + e.x) != ra) st_cg(p + e.x, ra);
    if (e.y != ra && ld_cg(p + e.y) != ra) st_cg(p + e.y, ra);
  }
}

// Row i of a stratified sample: a hashed position inside stratum i, so that
// a sample stride never aliases with a regular structure of the ids (grid rows).
__host__ __device__ __forceinline__ uint64_t sample_row(uint64_t i, uint64_t samples, uint64_t n) {
  const uint64_t lo = i * n / samples, hi = (i + 1) * n / samples;
  return hi > lo ? lo + mix64(0x9e3779b97f4a7c15ull ^ i) % (hi - lo) : lo;
}

// Sampled edges (u < v, same rank): total, edges leaving their tile, and edges
// of hub rows (about half of a hub row's entries are u < v).  Both kinds are
// left to global unions by the tiled pass.  Also the rows' link-round entries
// (the sampled-linking edges): total and leaving the tile.
template <class T, bool PART>
__global__ void k_cut_sample(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                             const T *__restrict__ col, PartMap pm, uint32_t tile,
                             uint32_t hub_degree, uint32_t samples,
                             unsigned long long *__restrict__ counts) {
  unsigned long long tot = 0, cross = 0, hub = 0, ltot = 0, lcross = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < samples; i += gridDim.x * blockDim.x) {
    uint64_t v = sample_row(i, samples, n);
    uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    if (e < b || e > m) continue;
    // the link-round entries of the row
    for (uint32_t r = 0; r < kAffRounds && r < e - b; ++r) {
      const uint64_t u = (uint64_t)__ldg(col + b + link_pos<PART>(v, e - b, r));
      if (u >= n || u == v) continue;
      ++ltot;
      lcross += u / tile != v / tile;
    }
    if (e - b > hub_degree) {
      tot += (e - b) / 2;
      hub += (e - b) / 2;
      continue;
    }
    uint64_t t0 = v / tile * tile;
    uint32_t lo = PART ? part_lo(pm, (uint32_t)v) : 0u;
    for (uint64_t k = b; k < e; ++k) {
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= v || u < lo) continue;
      ++tot;
      cross += u < t0;
    }
  }
  atomicAdd(counts, tot);
  atomicAdd(counts + 1, cross);
  atomicAdd(counts + 2, hub);
  atomicAdd(counts + 3, ltot);
  atomicAdd(counts + 4, lcross);
}

template <class OUT>
__global__ void k_widen(const uint32_t *__restrict__ in, OUT *__restrict__ out, uint64_t n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    out[v] = (OUT)in[v];
}

// The caller's offsets and ids checked (a bad one is recorded in the error
// word, and the solve stops before anything reads the graph again); 64-bit
// ids are also narrowed into a uint32 copy (out, else null).  Offsets and ids
// are two flat grid-stride loops: a hub row costs no more than any other
// stretch of entries.
template <class T>
__device__ __forceinline__ void sanitize_one(uint64_t k, uint64_t u, uint64_t n,
                                             uint32_t *__restrict__ out, int *err) {
  if (u >= n) set_err(err, kErrBadId);
  if (out) out[k] = (uint32_t)u;
}
template <class T>
__global__ void k_sanitize(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                           const T *__restrict__ col, uint32_t *__restrict__ out, int *err) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (uint64_t v = t; v < n; v += stride) {
    const uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    if (e < b || e > m) set_err(err, kErrBadOffsets);
  }
  // ids in 16-byte loads from the first 16-byte boundary on; the entries
  // before it and after the last whole vector one at a time
  constexpr uint64_t kVec = 16 / sizeof(T);
  const uint64_t mis = ((uintptr_t)col & 15) / sizeof(T);
  const uint64_t head = min(m, mis ? kVec - mis : 0);
  const uint64_t nvec = (m - head) / kVec;
  const uint4 *vcol = reinterpret_cast<const uint4 *>(col + head);
  for (uint64_t q = t; q < nvec; q += stride) {
    const uint4 w = __ldg(vcol + q);
    const T *x = reinterpret_cast<const T *>(&w);
    const uint64_t k0 = head + q * kVec;
#pragma unroll
    for (uint64_t j = 0; j < kVec; ++j) sanitize_one<T>(k0 + j, (uint64_t)x[j], n, out, err);
  }
  for (uint64_t k = t; k < head; k += stride) sanitize_one<T>(k, (uint64_t)__ldg(col + k), n, out, err);
  for (uint64_t k = head + nvec * kVec + t; k < m; k += stride)
    sanitize_one<T>(k, (uint64_t)__ldg(col + k), n, out, err);
}

template <class T, bool PART>
void run_uf(const Csr &g, uint32_t *parent, const PartMap &pm, uint32_t hub_degree,
            cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  const T *col = static_cast<const T *>(g.col);
  unsigned grid = grid_for(g.n, kBlock, num_sms() * 32);
  const uint64_t si = (uint64_t)g.idb;
  cudaEvent_t t0 = c.tic(s);
  k_init<T, PART><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_init", t0, 8 * (g.n + 1) + g.n * si + 4 * g.n);
  const uint64_t hub_cap = hub_list_cap(g.m, hub_degree);
  DevBuf hubs(8 * hub_cap, s, pool), nh(4, s, pool);
  CCG_CUDA(cudaMemsetAsync(nh.p, 0, 4, s));
  const HubList hl{hubs.as<uint2>(), hub_cap, nh.as<unsigned int>()};
  // hook: offsets, every id once, one parent gather per edge, own parent r/w
  const uint64_t hook_bytes = 8 * (g.n + 1) + g.m * si + g.m * 4 + 2 * g.n * 4;
  cudaEvent_t t1 = c.tic(s);
  k_hook<T, PART, PieceSink><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, hub_degree,
                                                    PieceSink{hl}, g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_hook", t1, hook_bytes);
  cudaEvent_t t2 = c.tic(s);
  // hub rows in pieces; every edge to a smaller id (the first one again too)
  k_hub_pieces<T, PART, true><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, hl,
                                                          g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_hook_hubs", t2, 0);
  cudaEvent_t t3 = c.tic(s);
  k_compress<<<grid_for(g.n, kBlock, num_sms() * 32), kBlock, 0, s>>>(g.n, parent);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_compress", t3, 3 * g.n * 4);
  c.add(4, (8 * (g.n + 1) + g.n * si + 4 * g.n) + hook_bytes + 3 * g.n * 4);
}

// Launch shape of the tile kernel: two CTAs per SM when the tile leaves room
// for a cut stage of at least 256 edges, else one; the stage takes what is
// left of the shared memory (at most 8192 edges).
struct TileShape {
  uint32_t tile = 0, stage = 0;
  int threads = 0;
  size_t smem = 0;
  unsigned grid = 0;
};
template <class T, bool PART, int LINK>
TileShape tile_shape_uncached(uint64_t n, const UfTuning &tu);

// The launch shape depends on the device, the tile and the CTA size only (the
// grid is clamped to the graph below); it is computed once per combination,
// because the attribute and occupancy queries cost more host time than a
// small solve.
template <class T, bool PART, int LINK>
TileShape tile_shape(uint64_t n, const UfTuning &tu) {
  static std::mutex mu;
  static std::map<std::tuple<int, uint32_t, uint32_t>, TileShape> cache;
  int dev = 0;
  CCG_CUDA(cudaGetDevice(&dev));
  const auto key = std::make_tuple(dev, tu.tile_vertices, tu.tile_threads);
  TileShape t;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) t = it->second;
  }
  if (t.threads == 0) {
    t = tile_shape_uncached<T, PART, LINK>(~0ull >> 1, tu);  // the widest grid for this shape
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = t;
  }
  const uint64_t tiles = (n + t.tile - 1) / t.tile;
  t.grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)t.grid);
  return t;
}

template <class T, bool PART, int LINK>
TileShape tile_shape_uncached(uint64_t n, const UfTuning &tu) {
  TileShape t;
  if (tu.tile_vertices < 32 || tu.tile_vertices > kTileMax)
    throw Error(CC_ERR_INVALID, "tile_vertices must lie in [32, 65536]");
  // link mode: 32-bit parents, half the vertices in the same shared memory
  t.tile = LINK > 0 ? std::max<uint32_t>(32, tu.tile_vertices / 2) : tu.tile_vertices;
  t.threads = (int)tu.tile_threads;
  if (t.threads < 32 || t.threads > 1024 || t.threads % 32)
    throw Error(CC_ERR_INVALID, "tile_threads must be a multiple of 32 up to 1024");
  int dev = 0, sm_smem = 0, blk_smem = 0;
  CCG_CUDA(cudaGetDevice(&dev));
  CCG_CUDA(cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  CCG_CUDA(cudaDeviceGetAttribute(&blk_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t fixed = tile_smem_bytes<TileParent<LINK>>(t.tile, (uint32_t)t.threads, 0);
  const size_t reserve = 1024 + 64;  // per-CTA system reserve + static shared memory
  size_t room = (size_t)sm_smem / 2 > reserve + fixed ? (size_t)sm_smem / 2 - reserve - fixed : 0;
  if (room < 256 * 8) room = (size_t)blk_smem > 64 + fixed ? (size_t)blk_smem - 64 - fixed : 0;
  t.stage = (uint32_t)std::min<size_t>(room / 8, 8192);
  if (t.stage < 64) throw Error(CC_ERR_INVALID, "tile does not fit in shared memory");
  t.smem = tile_smem_bytes<TileParent<LINK>>(t.tile, (uint32_t)t.threads, t.stage);
  const void *fn = (const void *)k_tile3<T, PART, TileParent<LINK>, LINK>;
  // the attribute only ever grows: launch shapes cached for other tiles keep working
  cudaFuncAttributes fa;
  CCG_CUDA(cudaFuncGetAttributes(&fa, fn));
  if ((size_t)fa.maxDynamicSharedSizeBytes < t.smem)
    CCG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t.smem));
  int per_sm = 0;
  CCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, t.threads, t.smem));
  if (per_sm < 1) throw Error(CC_ERR_INVALID, "tile does not fit in shared memory");
  const uint64_t tiles = (n + t.tile - 1) / t.tile;
  t.grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)per_sm * num_sms());
  return t;
}

// Final compression when the labels go to the caller's host uint32 array:
// compress in chunks and copy each chunk out on the copy stream as soon as it
// is final (a chunk's entries are written only by its own launch), so the
// device-to-host copy overlaps the later chunks.  All launches are queued
// first: a copy into pageable memory blocks the host.
void compress_copy_out(uint64_t n, uint32_t *parent, const HostSource *hs, cudaStream_t s,
                       Counters &c) {
  constexpr int kOutChunks = 8;
  const uint64_t step = ((n + kOutChunks - 1) / kOutChunks + 1023) / 1024 * 1024;
  cudaEvent_t done[kOutChunks];
  int nch = 0;
  cudaEvent_t t3 = c.tic(s);
  for (uint64_t a = 0; a < n; a += step, ++nch) {
    const uint64_t b = std::min<uint64_t>(n, a + step);
    k_compress<<<grid_for(b - a, kBlock, num_sms() * 32), kBlock, 0, s>>>(b, parent, a);
    CCG_LAUNCH_CHECK();
    CCG_CUDA(cudaEventCreateWithFlags(&done[nch], cudaEventDisableTiming));
    CCG_CUDA(cudaEventRecord(done[nch], s));
  }
  c.toc(s, "uf_compress", t3, 3 * n * 4);
  for (int k = 0; k < nch; ++k) {
    const uint64_t a = (uint64_t)k * step, b = std::min<uint64_t>(n, a + step);
    CCG_CUDA(cudaStreamWaitEvent(hs->copy, done[k], 0));
    CCG_CUDA(cudaMemcpyAsync(static_cast<uint32_t *>(hs->labels_out) + a, parent + a, 4 * (b - a),
                             cudaMemcpyDeviceToHost, hs->copy));
    cudaEventDestroy(done[k]);
  }
  cudaEvent_t copied;  // the caller's stream ends after the last copy
  CCG_CUDA(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming));
  CCG_CUDA(cudaEventRecord(copied, hs->copy));
  CCG_CUDA(cudaStreamWaitEvent(s, copied, 0));
  cudaEventDestroy(copied);
  c.add(nch - 1, 0);
}

// Staging of the row offsets of a streamed host CSR as degree bytes with
// escapes: one byte per row, 255 for rows of 255 entries or more, whose exact
// degrees follow as (row, degree) pairs.  Host side in page-locked memory
// (encoded by the context's host threads while the copy engine moves the
// previous chunk), device side in pool memory; each chunk's escapes take the
// next slice of the escape area.
struct DegreeStage {
  uint8_t *hdeg = nullptr;
  uint2 *hesc = nullptr;
  DevBuf ddeg, desc;
  uint64_t esc_used = 0, esc_cap = 0;
  DegreeStage(const Csr &g, const HostSource *hs, cudaStream_t s, cudaMemPool_t pool) {
    if (!hs->stager) return;
    esc_cap = g.m / 255 + 2;
    const uint64_t deg_bytes = (g.n + 15) / 16 * 16;
    uint8_t *base = hs->stager->staging(deg_bytes + 8 * esc_cap);
    if (!base) return;
    hdeg = base;
    hesc = reinterpret_cast<uint2 *>(base + deg_bytes);
    ddeg.alloc(g.n, s, pool);
    desc.alloc(8 * esc_cap, s, pool);
  }
  // Encode rows [v0, v1) (host threads); false when a degree does not fit 32
  // bits (offsets not monotone: the kernels report them) - send offsets.
  bool encode(const HostSource *hs, uint64_t v0, uint64_t v1, uint32_t *nesc) {
    if (!hdeg) return false;
    constexpr uint64_t kPart = 1 << 16;
    const unsigned parts = (unsigned)((v1 - v0 + kPart - 1) / kPart);
    std::vector<std::vector<uint2>> esc(parts);
    std::atomic<int> bad{0};
    hs->stager->pool.run(parts, [&](unsigned i) {
      const uint64_t a = v0 + (uint64_t)i * kPart, b = std::min<uint64_t>(v1, a + kPart);
      uint64_t prev = hs->rp[a];
      for (uint64_t v = a; v < b; ++v) {
        const uint64_t nx = hs->rp[v + 1], d = nx - prev;  // wraps to huge when not monotone
        prev = nx;
        if (d < 255) {
          hdeg[v] = (uint8_t)d;
        } else {
          hdeg[v] = 255;
          if (d >= (1ull << 32)) bad.store(1);
          esc[i].push_back(make_uint2((uint32_t)v, (uint32_t)d));
        }
      }
    });
    if (bad.load()) return false;
    uint64_t k = 0;
    for (auto &e : esc) k += e.size();
    if (esc_used + k > esc_cap) return false;
    uint2 *dst = hesc + esc_used;
    for (auto &e : esc)
      for (const uint2 &x : e) *dst++ = x;
    *nesc = (uint32_t)k;
    return true;
  }
};

// Copy rows [v0, v1) of the caller's host CSR (their offsets v0 .. v1 and
// their ids) into the device buffers of g on the copy stream, and make s wait
// for them.  With a degree stage, every chunk but the first sends its offsets
// as degree bytes with escapes and the device rebuilds them (the first goes as
// offsets, so that the copy engine starts at once).
template <class T>
void copy_rows_in(const Csr &g, const HostSource *hs, uint64_t v0, uint64_t v1, cudaStream_t s,
                  DegreeStage *ds = nullptr, cudaMemPool_t pool = nullptr, Counters *c = nullptr) {
  const uint64_t e0 = hs->rp[v0], e1 = hs->rp[v1];
  if (e1 < e0 || e1 > g.m) throw Error(CC_ERR_INVALID, "CSR offsets are not monotone or exceed m_dir");
  uint32_t nesc = 0;
  const uint64_t esc_at = ds ? ds->esc_used : 0;
  const bool coded = ds && v0 > 0 && e1 - e0 < (1ull << 32) && ds->encode(hs, v0, v1, &nesc);
  if (coded) {
    CCG_CUDA(cudaMemcpyAsync(ds->ddeg.as<uint8_t>() + v0, ds->hdeg + v0, v1 - v0,
                             cudaMemcpyHostToDevice, hs->copy));
    if (nesc)
      CCG_CUDA(cudaMemcpyAsync(ds->desc.as<uint2>() + esc_at, ds->hesc + esc_at, 8ull * nesc,
                               cudaMemcpyHostToDevice, hs->copy));
    ds->esc_used += nesc;
    hs->h2d_bytes += (v1 - v0) + 8ull * nesc;
  } else {
    CCG_CUDA(cudaMemcpyAsync(const_cast<uint64_t *>(g.rp) + v0, hs->rp + v0, 8 * (v1 - v0 + 1),
                             cudaMemcpyHostToDevice, hs->copy));
    hs->h2d_bytes += 8 * (v1 - v0 + 1);
  }
  if (!hs->in_place) {  // in place: the kernels read the ids from the caller's buffer
    if (e1 > e0)
      CCG_CUDA(cudaMemcpyAsync(const_cast<T *>(static_cast<const T *>(g.col)) + e0,
                               static_cast<const T *>(hs->col) + e0, sizeof(T) * (e1 - e0),
                               cudaMemcpyHostToDevice, hs->copy));
    hs->h2d_bytes += sizeof(T) * (e1 - e0);
  }
  cudaEvent_t ev;
  CCG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CCG_CUDA(cudaEventRecord(ev, hs->copy));
  CCG_CUDA(cudaStreamWaitEvent(s, ev, 0));
  cudaEventDestroy(ev);
  if (coded)
    offsets_from_degrees_esc(ds->ddeg.as<uint8_t>() + v0, v1 - v0, v0, e0, ds->desc.as<uint2>() + esc_at,
                             nesc, const_cast<uint64_t *>(g.rp) + v0, s, pool, *c);
}

template <class T, bool PART>
void run_uf_tiled(const Csr &g, uint32_t *parent, const PartMap &pm, const UfTuning &tu,
                  cudaStream_t s, cudaMemPool_t pool, Counters &c, const HostSource *hs) {
  const T *col = static_cast<const T *>(g.col);
  const uint64_t si = (uint64_t)g.idb;
  const TileShape ts = tile_shape<T, PART, 0>(g.n, tu);
  const uint32_t tile = ts.tile, stage = ts.stage;
  const int threads = ts.threads;
  const size_t smem = ts.smem;
  const unsigned grid = ts.grid;
  const uint64_t hub_cap = hub_list_cap(g.m, tu.hub_degree);
  const uint64_t cut_cap = g.m + 1;
  DevBuf hubs(8 * hub_cap, s, pool), nh(4, s, pool), cut(8 * cut_cap, s, pool), cnt(16, s, pool);
  const HubList hl{hubs.as<uint2>(), hub_cap, nh.as<unsigned int>()};
  CCG_CUDA(cudaMemsetAsync(nh.p, 0, 4, s));
  CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 16, s));
  unsigned long long *ncut = cnt.as<unsigned long long>();
  unsigned long long *united = ncut + 1;  // streamed input: cut edges united so far
  // tile pass: offsets, every id once, own parent written once (the parent
  // chains stay in shared memory); cut edges are counted where read
  const uint64_t tile_bytes = 8 * (g.n + 1) + g.m * si + 4 * g.n;
  cudaEvent_t t0 = c.tic(s);
  if (!hs) {
    k_tile3<T, PART, TileParent<0>, 0><<<grid, threads, smem, s>>>(g.n, g.m, 0, g.n, g.rp, col, parent,
                                                           pm, tile, stage, tu.hub_degree, hl,
                                                           cut.as<uint2>(), cut_cap, ncut, g.err);
    CCG_LAUNCH_CHECK();
  } else {
    // Copy tile-aligned chunks of the caller's host CSR on the copy stream and
    // run each chunk's tiles as soon as its slice is on the device: the tile
    // pass overlaps the host-to-device transfer.  A chunk's cut edges lead to
    // earlier tiles only, so they are united right after its tiles (later
    // tiles never touch those entries), and only the last chunk's remain once
    // the transfer ends.
    // Rows are sent as one degree byte each when every row of the chunk has
    // fewer than 255 entries (the host threads encode the next chunk while
    // the copy engine moves this one; the device rebuilds the offsets with a
    // prefix sum), else as their 8-byte offsets.  The first chunk always goes
    // as offsets: the copy engine starts at once, and the encoding of the
    // later chunks (host threads) and the copies (host link) then run side by
    // side.
    const uint64_t chunk = (uint64_t)grid * tile;  // one full wave of CTAs
    uint8_t *hdeg = hs->stager ? hs->stager->staging(g.n) : nullptr;
    DevBuf ddeg;
    if (hdeg) ddeg.alloc(g.n, s, pool);
    uint64_t *drp = const_cast<uint64_t *>(g.rp);
    for (uint64_t v0 = 0; v0 < g.n; v0 += chunk) {
      const uint64_t v1 = std::min<uint64_t>(g.n, v0 + chunk);
      const uint64_t e0 = hs->rp[v0], e1 = hs->rp[v1];
      if (e1 < e0 || e1 > g.m) throw Error(CC_ERR_INVALID, "CSR offsets are not monotone or exceed m_dir");
      bool coded = false;
      if (hdeg && v0 > 0 && e1 - e0 < (1ull << 32)) {
        constexpr uint64_t kPart = 1 << 16;
        std::atomic<int> wide{0};
        hs->stager->pool.run((unsigned)((v1 - v0 + kPart - 1) / kPart), [&](unsigned i) {
          const uint64_t a = v0 + (uint64_t)i * kPart, b = std::min<uint64_t>(v1, a + kPart);
          uint64_t prev = hs->rp[a], mx = 0;
          for (uint64_t v = a; v < b; ++v) {
            const uint64_t nx = hs->rp[v + 1], d = nx - prev;  // wraps to huge when not monotone
            mx = d > mx ? d : mx;
            hdeg[v] = (uint8_t)d;
            prev = nx;
          }
          if (mx >= 255) wide.store(1);
        });
        coded = wide.load() == 0;
      }
      if (coded)
        CCG_CUDA(cudaMemcpyAsync(ddeg.as<uint8_t>() + v0, hdeg + v0, v1 - v0, cudaMemcpyHostToDevice,
                                 hs->copy));
      else
        CCG_CUDA(cudaMemcpyAsync(drp + v0, hs->rp + v0, 8 * (v1 - v0 + 1), cudaMemcpyHostToDevice,
                                 hs->copy));
      hs->h2d_bytes += (coded ? v1 - v0 : 8 * (v1 - v0 + 1)) + si * (e1 - e0);
      if (e1 > e0)
        CCG_CUDA(cudaMemcpyAsync(static_cast<char *>(const_cast<void *>(g.col)) + si * e0,
                                 static_cast<const char *>(hs->col) + si * e0, si * (e1 - e0),
                                 cudaMemcpyHostToDevice, hs->copy));
      cudaEvent_t ev;
      CCG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      CCG_CUDA(cudaEventRecord(ev, hs->copy));
      CCG_CUDA(cudaStreamWaitEvent(s, ev, 0));
      cudaEventDestroy(ev);
      if (coded) offsets_from_degrees(ddeg.as<uint8_t>() + v0, v1 - v0, e0, drp + v0, s, pool, c);
      const unsigned cgrid = (unsigned)std::min<uint64_t>((v1 - v0 + tile - 1) / tile, grid);
      k_tile3<T, PART, TileParent<0>, 0><<<cgrid, threads, smem, s>>>(g.n, g.m, v0, v1, g.rp, col,
                                                              parent, pm, tile, stage,
                                                              tu.hub_degree, hl, cut.as<uint2>(),
                                                              cut_cap, ncut, g.err);
      CCG_LAUNCH_CHECK();
      k_cut_union<<<num_sms() * kCutCtasTiled, kBlock, 0, s>>>(cut.as<uint2>(), ncut, cut_cap, parent, united);
      CCG_LAUNCH_CHECK();
      CCG_CUDA(cudaMemcpyAsync(united, ncut, 8, cudaMemcpyDeviceToDevice, s));
    }
  }
  c.toc(s, hs ? "uf_tile_streamed" : "uf_tile", t0, tile_bytes);
  if (!hs) {
    cudaEvent_t t1 = c.tic(s);
    k_cut_union<<<num_sms() * kCutCtasTiled, kBlock, 0, s>>>(cut.as<uint2>(), ncut, cut_cap, parent);
    CCG_LAUNCH_CHECK();
    c.toc(s, "uf_cut_union", t1, 0);
  }
  cudaEvent_t t2 = c.tic(s);
  k_hub_pieces<T, PART, true><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm,
                                                          hl, g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_hook_hubs", t2, 0);
  // every vertex points at a tile-local root or at a final root: full
  // compression, writing only the entries that change
  if (hs && hs->labels_out) {
    compress_copy_out(g.n, parent, hs, s, c);
  } else {
    cudaEvent_t t3 = c.tic(s);
    k_compress<<<grid_for(g.n, kBlock, num_sms() * 32), kBlock, 0, s>>>(g.n, parent);
    CCG_LAUNCH_CHECK();
    c.toc(s, "uf_compress", t3, 3 * g.n * 4);
  }
  c.add(4, tile_bytes + 3 * g.n * 4);
}

// The tiled pass suits a graph when a sample of rows shows fewer than half of
// the edges leaving their tile and fewer than a tenth in hub rows (hub edges
// contend on a few global roots; the sampled pass skips most of them).
inline bool tiles_fit(uint64_t tot, uint64_t cross, uint64_t hub) {
  return tot == 0 || (2 * cross < tot && 10 * hub < tot);
}

// Both decisions on a sample of 8192 rows of a device graph (one small
// readback): the tiled pass, and whether the link rounds of sampled linking
// run as a tiled pass (at least three quarters of their edges in the tile).
struct Shares {
  bool tiles = false, link_tiles = false, few_hubs = true;
};
template <class T, bool PART>
Shares sample_shares(const Csr &g, const PartMap &pm, uint32_t tile, uint32_t hub_degree,
                     cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  DevBuf cnt(40, s, pool);
  CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 40, s));
  const uint32_t samples = (uint32_t)std::min<uint64_t>(g.n, 8192);
  k_cut_sample<T, PART><<<(samples + 255) / 256, 256, 0, s>>>(
      g.n, g.m, g.rp, static_cast<const T *>(g.col), pm, tile, hub_degree, samples,
      cnt.as<unsigned long long>());
  CCG_LAUNCH_CHECK();
  unsigned long long h[5] = {0, 0, 0, 0, 0};
  CCG_CUDA(cudaMemcpyAsync(h, cnt.p, 40, cudaMemcpyDeviceToHost, s));
  CCG_CUDA(cudaStreamSynchronize(s));
  c.add(1, 0);
  Shares r;
  r.tiles = tiles_fit(h[0], h[1], h[2]);
  r.link_tiles = h[3] > 0 && 4 * h[4] < h[3];
  r.few_hubs = 10 * h[2] < h[0] || h[0] == 0;
  return r;
}

template <class T, bool PART>
void run_uf_afforest(const Csr &g, uint32_t *parent, const PartMap &pm, const UfTuning &tu,
                     bool link_tiles, cudaStream_t s, cudaMemPool_t pool, Counters &c,
                     const HostSource *hs = nullptr) {
  const T *col = static_cast<const T *>(g.col);
  const uint64_t si = (uint64_t)g.idb;
  const uint32_t hub_degree = tu.hub_degree;
  const unsigned grid = grid_for(g.n, kBlock, num_sms() * 32);
  uint64_t link_bytes = 0;
  if (link_tiles) {
    // link rounds as one tiled pass: the link-round entries of every row,
    // united in shared memory when they stay in the tile (most do on
    // geometric and angularly ordered graphs), the others as cut edges
    const TileShape ts = tile_shape<T, PART, (int)kAffRounds>(g.n, tu);
    const uint64_t cut_cap = std::min<uint64_t>(g.m, kAffRounds * g.n) + 1;
    DevBuf cut(8 * cut_cap, s, pool), cnt(8, s, pool);
    CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 8, s));
    const HubList none{nullptr, 0, nullptr};  // no row is queued in link mode
    // offsets, the link-round ids, own parent
    link_bytes = 8 * (g.n + 1) + kAffRounds * g.n * si + 4 * g.n;
    cudaEvent_t t0 = c.tic(s);
    if (!hs || (hs->in_place && !hs->offsets_copied)) {
      // host buffers read in place: the pass reads each row's offsets and link
      // entries across the host link, the only ids most rows ever need (the
      // remaining pass reads the rows outside the giant component)
      k_tile3<T, PART, TileParent<(int)kAffRounds>, (int)kAffRounds><<<ts.grid, ts.threads, ts.smem, s>>>(
          g.n, g.m, 0, g.n, g.rp, col, parent, pm, ts.tile, ts.stage, hub_degree, none,
          cut.as<uint2>(), cut_cap, cnt.as<unsigned long long>(), g.err);
      CCG_LAUNCH_CHECK();
    } else {
      // host input: tile-aligned chunks of rows cross the host link on the
      // copy stream, and each chunk's tiles are linked as soon as it has
      // landed, so the link pass runs under the transfer.  Link edges may
      // lead to later tiles, so every cut edge waits for the cut union after
      // the last chunk (a tile writes its vertices' parents when it ends).
      const uint64_t chunk = (uint64_t)ts.grid * ts.tile;  // one full wave of CTAs
      DegreeStage ds(g, hs, s, pool);
      for (uint64_t v0 = 0; v0 < g.n; v0 += chunk) {
        const uint64_t v1 = std::min<uint64_t>(g.n, v0 + chunk);
        copy_rows_in<T>(g, hs, v0, v1, s, &ds, pool, &c);
        const unsigned cgrid = (unsigned)std::min<uint64_t>((v1 - v0 + ts.tile - 1) / ts.tile, ts.grid);
        k_tile3<T, PART, TileParent<(int)kAffRounds>, (int)kAffRounds><<<cgrid, ts.threads, ts.smem, s>>>(
            g.n, g.m, v0, v1, g.rp, col, parent, pm, ts.tile, ts.stage, hub_degree, none,
            cut.as<uint2>(), cut_cap, cnt.as<unsigned long long>(), g.err);
        CCG_LAUNCH_CHECK();
      }
    }
    c.toc(s,
          !hs                   ? "uf_sample_link_tiled"
          : !hs->in_place       ? "uf_sample_link_streamed"
          : hs->offsets_copied  ? "uf_sample_link_ids_in_place"
                                : "uf_sample_link_in_place",
          t0, link_bytes);
    // in place: up to kAffRounds link entries a row, and the offsets unless
    // they were copied (the link moves whole sectors around the entries)
    if (hs && hs->in_place)
      hs->h2d_bytes = (hs->offsets_copied ? hs->h2d_bytes : 8 * (g.n + 1)) +
                      std::min<uint64_t>(g.m, kAffRounds * g.n) * si;
    cudaEvent_t t1 = c.tic(s);
    k_cut_union<<<num_sms() * kCutCtasLink, kBlock, 0, s>>>(cut.as<uint2>(), cnt.as<unsigned long long>(),
                                             cut_cap, parent);
    CCG_LAUNCH_CHECK();
    c.toc(s, "uf_cut_union", t1, 0);
  } else {
    k_iota_parent<<<grid, kBlock, 0, s>>>(g.n, parent);
    CCG_LAUNCH_CHECK();
    // each link round: offsets, one id, one union (two parent gathers); the
    // rounds stay separate launches (one round's links all land before the
    // next round's finds, which keeps the trees shallow)
    const uint64_t round_bytes = 8 * (g.n + 1) + g.n * (si + 2 * 4);
    for (uint32_t r = 0; r < kAffRounds; ++r) {
      cudaEvent_t t0 = c.tic(s);
      k_aff_link<T, PART><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, r, g.err);
      CCG_LAUNCH_CHECK();
      c.toc(s, "uf_sample_link", t0, round_bytes);
    }
    link_bytes = kAffRounds * round_bytes;
  }
  k_compress<<<grid_for(g.n, kBlock, num_sms() * 32), kBlock, 0, s>>>(g.n, parent);
  CCG_LAUNCH_CHECK();
  // most frequent root of a sample = the giant component, if there is one;
  // with virtual ranks (up to 4096) one per rank, as each rank has its own
  // giant local component
  uint32_t P = 1;
  if (PART) P = pm.q ? pm.rm + (uint32_t)((g.n - pm.big) / pm.q) : (uint32_t)g.n;
  const uint32_t nparts = (PART && P > 1 && P <= 4096) ? P : 1;
  const uint32_t per = nparts > 1 ? 64u : (uint32_t)std::min<uint64_t>(g.n, 1024);
  const uint32_t samples = nparts * per;
  DevBuf smp(4 * samples, s, pool), dL(4 * nparts, s, pool);
  k_aff_sample<<<(samples + 255) / 256, 256, 0, s>>>(g.n, parent, pm, nparts, per, 0x5eedull,
                                                     smp.as<uint32_t>());
  CCG_LAUNCH_CHECK();
  // the mode of each partition's samples, on the device (no host round trip)
  k_aff_mode<<<nparts, kModeBlock, 0, s>>>(smp.as<uint32_t>(), per, dL.as<uint32_t>());
  CCG_LAUNCH_CHECK();
  const uint64_t hub_cap = hub_list_cap(g.m, hub_degree);
  DevBuf hubs(8 * hub_cap, s, pool), nh(4, s, pool);
  CCG_CUDA(cudaMemsetAsync(nh.p, 0, 4, s));
  const HubList hl{hubs.as<uint2>(), hub_cap, nh.as<unsigned int>()};
  // remaining pass: every row's root; then, for the rows outside the giant
  // component, offsets and one id and one root gather per remaining edge.  The
  // edge part is counted on the device while profiling and left out otherwise.
  uint64_t rest_bytes = 4 * g.n;
  DevBuf ecount(16, s, pool);
  if (c.prof) CCG_CUDA(cudaMemsetAsync(ecount.p, 0, 16, s));
  cudaEvent_t t1 = c.tic(s);
  k_aff_rest<T, PART><<<grid, kBlock, 0, s>>>(
      g.n, g.m, g.rp, col, parent, pm, dL.as<uint32_t>(), nparts, hub_degree, hl, g.err,
      c.prof ? ecount.as<unsigned long long>() : nullptr);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_sample_rest", t1, rest_bytes);
  if (c.prof && !c.recs.empty()) {
    unsigned long long cnt[2] = {0, 0};  // ids read, rows whose offsets were read
    CCG_CUDA(cudaMemcpyAsync(cnt, ecount.p, 16, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    rest_bytes += cnt[0] * (si + 4) + cnt[1] * 16;
    c.recs.back().bytes = rest_bytes;
  }
  cudaEvent_t th = c.tic(s);
  k_hub_pieces<T, PART, false><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, hl,
                                                           g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_sample_hubs", th, 0);
  if (hs && hs->labels_out) {
    compress_copy_out(g.n, parent, hs, s, c);
  } else {
    cudaEvent_t t2 = c.tic(s);
    k_compress<<<grid_for(g.n, kBlock, num_sms() * 32), kBlock, 0, s>>>(g.n, parent);
    CCG_LAUNCH_CHECK();
    c.toc(s, "uf_compress", t2, 3 * g.n * 4);
  }
  c.add((link_tiles ? 2 : 1 + kAffRounds) + 6, link_bytes + rest_bytes + 6 * g.n * 4);
}

// Working set (offsets, ids, parents) that the 129 MB L2 keeps resident
// during a hook pass, with room for the other streams' lines.
constexpr uint64_t kL2Resident = 96ull << 20;

template <class T, bool PART>
void run_uf_mode(const Csr &g, uint32_t *parent, const PartMap &pm, const UfTuning &tu,
                 cudaStream_t s, cudaMemPool_t pool, Counters &c, const HostSource *hs) {
  if (hs) {  // the caller decided on the host: the tiled pass, or sampled linking
    // with tiled link rounds, both streamed under the host-to-device copy
    if (hs->sampled) run_uf_afforest<T, PART>(g, parent, pm, tu, true, s, pool, c, hs);
    else run_uf_tiled<T, PART>(g, parent, pm, tu, s, pool, c, hs);
    return;
  }
  int mode = tu.mode;
  const bool big = g.n >= 4ull * tu.tile_vertices;
  Shares sh;
  if (big && (mode == kUfAuto || (mode == kUfSampled && tu.link_tiles < 0))) {
    UfDecisionCache *dc = tu.cache;
    const uint64_t parts_key = ((uint64_t)pm.q << 32) ^ pm.rm ^ ((uint64_t)PART << 63);
    if (dc && dc->valid && dc->rp == g.rp && dc->col == g.col && dc->n == g.n && dc->m == g.m &&
        dc->parts_key == parts_key && dc->tile == tu.tile_vertices && dc->hub == tu.hub_degree) {
      sh.tiles = dc->tiles;
      sh.link_tiles = dc->link_tiles;
      sh.few_hubs = dc->few_hubs;
    } else {
      sh = sample_shares<T, PART>(g, pm, tu.tile_vertices, tu.hub_degree, s, pool, c);
      if (dc) {
        dc->rp = g.rp;
        dc->col = g.col;
        dc->n = g.n;
        dc->m = g.m;
        dc->parts_key = parts_key;
        dc->tile = tu.tile_vertices;
        dc->hub = tu.hub_degree;
        dc->tiles = sh.tiles;
        dc->link_tiles = sh.link_tiles;
        dc->few_hubs = sh.few_hubs;
        dc->valid = true;
      }
    }
  }
  if (tu.link_tiles >= 0) sh.link_tiles = big && tu.link_tiles > 0;
  // the tiled pass wins when most edges stay inside their tile and few lie in
  // hub rows (grids, geometric graphs); a graph that L2 holds and that has few
  // hub rows is linked fastest by the plain global hook (every access an L2
  // hit, no sampling rounds); otherwise sampled linking
  if (mode == kUfAuto) {
    const uint64_t ws = 8 * (g.n + 1) + g.m * (uint64_t)g.idb + 4 * g.n;
    if (big && sh.tiles) mode = kUfTiled;
    else if (ws <= kL2Resident && sh.few_hubs) mode = kUfGlobal;
    else mode = kUfSampled;
  }
  if (mode == kUfTiled) run_uf_tiled<T, PART>(g, parent, pm, tu, s, pool, c, nullptr);
  else if (mode == kUfSampled) run_uf_afforest<T, PART>(g, parent, pm, tu, sh.link_tiles, s, pool, c);
  else run_uf<T, PART>(g, parent, pm, tu.hub_degree, s, pool, c);
}

}  // namespace

void uf_components(const Csr &g, uint32_t *parent, const PartMap *pm, const UfTuning &tu_in,
                   cudaStream_t s, cudaMemPool_t pool, Counters &c, const HostSource *hs) {
  if (g.n == 0) return;
  UfTuning tu = tu_in;
  if (tu.hub_degree < 1) tu.hub_degree = 32;
  if (tu.tile_vertices == 0) tu.tile_vertices = 16384;
  if (tu.tile_threads == 0) tu.tile_threads = 1024;
  PartMap p = pm ? *pm : PartMap(g.n, 1);
  bool part = pm != nullptr && !(pm->rm == 0 && pm->q == g.n);
  if (g.idb == 8) {
    if (part) run_uf_mode<uint64_t, true>(g, parent, p, tu, s, pool, c, hs);
    else run_uf_mode<uint64_t, false>(g, parent, p, tu, s, pool, c, hs);
  } else {
    if (part) run_uf_mode<uint32_t, true>(g, parent, p, tu, s, pool, c, hs);
    else run_uf_mode<uint32_t, false>(g, parent, p, tu, s, pool, c, hs);
  }
}

HostShares host_shares(const uint64_t *rp, const void *col, int idb, uint64_t n, uint64_t m,
                       uint32_t tile, uint32_t hub_degree, uint64_t max_samples) {
  const uint64_t samples = std::min<uint64_t>(n, max_samples);
  uint64_t tot = 0, cross = 0, hub = 0, ltot = 0, lcross = 0;
  auto id = [&](uint64_t k) -> uint64_t {
    return idb == 8 ? static_cast<const uint64_t *>(col)[k] : static_cast<const uint32_t *>(col)[k];
  };
  for (uint64_t i = 0; i < samples; ++i) {
    const uint64_t v = sample_row(i, samples, n), t0 = v / tile * tile;
    const uint64_t b = rp[v], e = rp[v + 1];
    if (e < b || e > m) continue;  // malformed rows are reported by the kernels
    for (uint32_t r = 0; r < kAffRounds && r < e - b; ++r) {
      const uint64_t u = id(b + link_pos<false>(v, e - b, r));  // one rank
      if (u >= n || u == v) continue;
      ++ltot;
      lcross += u / tile != v / tile;
    }
    if (e - b > hub_degree) {  // hub rows are united globally
      tot += (e - b) / 2;
      hub += (e - b) / 2;
      continue;
    }
    for (uint64_t k = b; k < e; ++k) {
      const uint64_t u = id(k);
      if (u >= v) continue;
      ++tot;
      cross += u < t0;
    }
  }
  HostShares r;
  r.tiles = tiles_fit(tot, cross, hub);
  r.link_tiles = ltot > 0 && 4 * lcross < ltot;
  r.few_hubs = tot == 0 || 10 * hub < tot;
  return r;
}

void widen_labels(const uint32_t *in, void *out, int out_bytes, uint64_t n, cudaStream_t s,
                  Counters &c) {
  if (n == 0) return;
  unsigned grid = grid_for(n, kBlock, num_sms() * 32);
  if (out_bytes == 8)
    k_widen<uint64_t><<<grid, kBlock, 0, s>>>(in, static_cast<uint64_t *>(out), n);
  else
    k_widen<uint32_t><<<grid, kBlock, 0, s>>>(in, static_cast<uint32_t *>(out), n);
  CCG_LAUNCH_CHECK();
  c.add(1, n * 4 + n * (uint64_t)out_bytes);
}

__global__ void k_check_offsets(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    if (e < b || e > m) set_err(err, kErrBadOffsets);
  }
}

void check_offsets(const Csr &g, cudaStream_t s, Counters &c) {
  if (g.n == 0) return;
  cudaEvent_t t0 = c.tic(s);
  k_check_offsets<<<grid_for(g.n, kBlock, num_sms() * 32), kBlock, 0, s>>>(g.n, g.m, g.rp, g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "check_offsets", t0, 8 * (g.n + 1));
  c.add(1, 8 * (g.n + 1));
}

void sanitize_ids(const Csr &g, uint32_t *col32, cudaStream_t s, Counters &c) {
  if (g.n == 0) return;
  unsigned grid = grid_for(std::max(g.n, g.m / 4), kBlock, num_sms() * 32);
  cudaEvent_t t0 = c.tic(s);
  if (g.idb == 8)
    k_sanitize<uint64_t><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp,
                                                 static_cast<const uint64_t *>(g.col), col32, g.err);
  else
    k_sanitize<uint32_t><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp,
                                                 static_cast<const uint32_t *>(g.col), col32, g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "check_ids", t0, 8 * (g.n + 1) + g.m * ((uint64_t)g.idb + (col32 ? 4 : 0)));
  c.add(1, 8 * (g.n + 1) + g.m * ((uint64_t)g.idb + (col32 ? 4 : 0)));
}

}  // namespace ccg

// ============================================================================
// Allocation-free entry point: cc_gpu_run_noalloc (declared in cc_gpu.h).
//
// Some callers cannot allocate device memory at the moment they need a
// solve: a plugin's enqueue() inside an inference runtime must not allocate,
// a process whose device memory is pre-reserved by its own allocator has
// nothing left for ours, and a latency-critical loop cannot afford the
// implicit device synchronisation of cudaMalloc/cudaFree.  This variant of
// the hook-and-compress solve therefore takes every buffer from the caller
// (CSR in, labels out, all on the device) and keeps its only scratch - the
// hub-row list, the hub counter and the error word - in the fixed array
// below, which every GPU that loads this library holds until the process
// exits.  It calls no cudaMalloc, cudaFree or any other allocating routine.
//
// Limits: the hub list holds kNoAllocHubCap rows of degree > 32, so a graph
// is accepted only if it cannot have more such rows:
//     min(n, m_dir / 33 + 1) <= kNoAllocHubCap   (1,048,512)
// e.g. any graph with n <= 1,048,512, or with m_dir <= 34.6 million.  Larger
// graphs get CC_ERR_UNSUPPORTED before anything is launched.
//
// Shared state: all calls share the one scratch array, and it keeps the last
// call's contents.  The counter and error word are cleared at the start of
// every call; calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.
//
// The call is synchronous: it waits on the caller's stream for the error word
// before it returns.
//
// Set-up: the first call on a device looks up the device address of the
// scratch array (cudaGetSymbolAddress) with that device current, and it is
// also the first launch of these kernels on that device, so CUDA's lazy
// module loading may allocate and synchronise during it.  Make one warm-up
// call per device before the point where allocation is forbidden, and before
// any stream capture begins on that device.
// ============================================================================
#include <algorithm>
#include <mutex>

namespace {

constexpr uint32_t kNoAllocWords = 1u << 20;                  // 4 MiB
constexpr uint32_t kNoAllocHeader = 64;                       // counter, error word, padding
constexpr uint32_t kNoAllocHubCap = kNoAllocWords - kNoAllocHeader;
constexpr uint32_t kNoAllocHubDegree = 32;
// The entry guard admits a graph only if min(n, m_dir / (kNoAllocHubDegree + 1)
// + 1) <= kNoAllocHubCap: a graph has at most m_dir / (degree + 1) rows above
// the hub degree, so the hub list cannot overflow.  An overflow word
// (kErrOverflow) would therefore mean a broken guard, reported as
// CC_ERR_UNSUPPORTED, not as bad caller input.
static_assert(kNoAllocHeader + kNoAllocHubCap <= kNoAllocWords, "hub list outside the scratch");
static_assert(kNoAllocHeader >= 2, "the header holds the hub counter and the error word");

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

constexpr int kNoAllocMaxDevices = 64;
uint32_t *g_noalloc_addr[kNoAllocMaxDevices] = {};
std::mutex g_noalloc_mu;

// Device address of the scratch array on the current device (looked up once
// per device; the host-side symbol itself is not a device address).
int noalloc_scratch(uint32_t **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CC_ERR_CUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return CC_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CC_ERR_CUDA;
    g_noalloc_addr[dev] = static_cast<uint32_t *>(p);
  }
  *out = g_noalloc_addr[dev];
  return CC_OK;
}

}  // namespace

extern "C" int cc_gpu_run_noalloc(const uint64_t *row_ptr, const uint32_t *col, uint64_t n,
                                  uint64_t m_dir, uint32_t *labels_out, void *stream) {
  using namespace ccg;
  if (n == 0) return CC_OK;
  if (!row_ptr || !labels_out || (m_dir > 0 && !col)) return CC_ERR_INVALID;
  if (n >= 0xffffffffull) return CC_ERR_UNSUPPORTED;
  const uint64_t worst_hubs = std::min<uint64_t>(n, m_dir / (kNoAllocHubDegree + 1) + 1);
  if (worst_hubs > kNoAllocHubCap) return CC_ERR_UNSUPPORTED;
  uint32_t *scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != CC_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned int *nhubs = scratch;                  // word 0
  int *err = reinterpret_cast<int *>(scratch + 1);  // word 1
  uint32_t *hubs = scratch + kNoAllocHeader;
  if (cudaMemsetAsync(scratch, 0, 2 * sizeof(uint32_t), s) != cudaSuccess) return CC_ERR_CUDA;
  const PartMap pm(n, 1);
  const unsigned grid = grid_for(n, kBlock, num_sms() * 32);
  k_init<uint32_t, false><<<grid, kBlock, 0, s>>>(n, m_dir, row_ptr, col, labels_out, pm, err);
  k_hook<uint32_t, false, RowSink><<<grid, kBlock, 0, s>>>(
      n, m_dir, row_ptr, col, labels_out, pm, kNoAllocHubDegree,
      RowSink{hubs, kNoAllocHubCap, nhubs}, err);
  k_hook_hubs<uint32_t, false><<<num_sms() * 8, kBlock, 0, s>>>(n, row_ptr, col, labels_out, pm, hubs,
                                                           kNoAllocHubCap, nhubs, err);
  k_compress<<<grid, kBlock, 0, s>>>(n, labels_out);
  if (cudaGetLastError() != cudaSuccess) return CC_ERR_CUDA;
  int host_err = 0;
  if (cudaMemcpyAsync(&host_err, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return CC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return CC_ERR_CUDA;
  if (host_err == kErrOverflow) return CC_ERR_UNSUPPORTED;
  return host_err ? CC_ERR_INVALID : CC_OK;
}

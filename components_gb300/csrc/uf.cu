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

#include "kernels.h"

namespace ccg {
namespace {

// Root of v with path halving.  parent[] only ever decreases along a path, so
// a stale read still names an ancestor; writes only shorten paths.
__device__ __forceinline__ uint32_t uf_find(uint32_t *p, uint32_t v) {
  uint32_t cur = ld_cg(p + v);
  if (cur == v) return v;
  uint32_t prev = v;
  uint32_t next;
  while (cur > (next = ld_cg(p + cur))) {
    st_cg(p + prev, next);
    prev = cur;
    cur = next;
  }
  return cur;
}

// Link the trees of a and b: the larger root is CAS'ed under the smaller one.
__device__ __forceinline__ void uf_union(uint32_t *p, uint32_t a, uint32_t b) {
  uint32_t ra = uf_find(p, a), rb = uf_find(p, b);
  while (ra != rb) {
    if (ra < rb) {
      uint32_t t = ra;
      ra = rb;
      rb = t;
    }
    uint32_t old = atomicCAS(p + ra, ra, rb);
    if (old == ra) return;
    ra = uf_find(p, old);
    rb = uf_find(p, rb);
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
      bool ok = u < v;
      if (PART && ok) ok = (uint32_t)u >= part_lo(pm, (uint32_t)v);
      if (ok) par = (uint32_t)u;
    }
    p[v] = par;
  }
}

template <class T, bool PART>
__global__ void k_hook(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                       const T *__restrict__ col, uint32_t *p, PartMap pm, uint32_t hub_degree,
                       uint32_t *__restrict__ hubs, uint64_t hub_cap,
                       unsigned int *__restrict__ nhubs, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    Row r;
    if (!load_row(rp, v, m, err, r)) continue;
    if (r.e - r.b > hub_degree) {
      uint32_t slot = atomicAdd(nhubs, 1u);
      if (slot < hub_cap) hubs[slot] = (uint32_t)v;
      else set_err(err, kErrOverflow);
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

// Full compression: parent[v] <- root.  Runs after every link is made.
__global__ void k_compress(uint64_t n, uint32_t *p) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t r = p[v];
    if (r == (uint32_t)v) continue;
    uint32_t nx;
    while ((nx = ld_cg(p + r)) != r) r = nx;
    p[v] = r;
  }
}

// ---- sampled linking (Afforest: Sutton, Ben-Nun, Barak, IPDPS 2018) ------------
// Link every vertex to its r-th neighbour for r < kAffRounds, compress, find
// the most frequent root L on a sample, then only vertices outside L's tree
// process their remaining edges.  An edge skipped by an endpoint inside L is
// either processed from its other endpoint or joins two vertices that are
// already connected, so the components are exact.  On graphs with a giant
// component most edges are never touched; without one it costs two light
// passes.
constexpr uint32_t kAffRounds = 2;

__device__ __forceinline__ bool same_part(const PartMap &pm, uint32_t v, uint32_t u) {
  return pm.part(v) == pm.part(u);
}

template <class T, bool PART>
__global__ void k_aff_link(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                           const T *__restrict__ col, uint32_t *p, PartMap pm, uint32_t r, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    Row row;
    if (!load_row(rp, v, m, err, row) || row.e - row.b <= r) continue;
    uint64_t u = (uint64_t)__ldg(col + row.b + r);
    if (u >= n) {
      set_err(err, kErrBadId);
      continue;
    }
    if (!PART || same_part(pm, (uint32_t)v, (uint32_t)u)) uf_union(p, (uint32_t)v, (uint32_t)u);
  }
}

__global__ void k_aff_sample(uint64_t n, const uint32_t *p, uint32_t samples, uint64_t salt,
                             uint32_t *__restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < samples; i += gridDim.x * blockDim.x) {
    uint32_t r = (uint32_t)(mix64(salt + i) % n), nx;
    while ((nx = ld_cg(p + r)) != r) r = nx;
    out[i] = r;
  }
}

template <class T, bool PART>
__global__ void k_aff_rest(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                           const T *__restrict__ col, uint32_t *p, PartMap pm, uint32_t L,
                           uint32_t hub_degree, uint32_t *__restrict__ hubs, uint64_t hub_cap,
                           unsigned int *__restrict__ nhubs, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    Row row;
    if (!load_row(rp, v, m, err, row) || row.e - row.b <= kAffRounds) continue;
    if (uf_find(p, (uint32_t)v) == L) continue;
    if (row.e - row.b > hub_degree) {
      uint32_t slot = atomicAdd(nhubs, 1u);
      if (slot < hub_cap) hubs[slot] = (uint32_t)v;
      else set_err(err, kErrOverflow);
      continue;
    }
    for (uint64_t k = row.b + kAffRounds; k < row.e; ++k) {
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        continue;
      }
      if (!PART || same_part(pm, (uint32_t)v, (uint32_t)u)) uf_union(p, (uint32_t)v, (uint32_t)u);
    }
  }
}

template <class T, bool PART>
__global__ void k_aff_rest_hubs(uint64_t n, const uint64_t *__restrict__ rp,
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
    uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);  // checked by k_aff_rest
    for (uint64_t k = b + kAffRounds + lane; k < e; k += 32) {
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        continue;
      }
      if (!PART || same_part(pm, v, (uint32_t)u)) uf_union(p, v, (uint32_t)u);
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
__device__ __forceinline__ uint32_t ts_find(volatile uint32_t *p, uint32_t v) {
  uint32_t cur = p[v];
  if (cur == v) return v;
  uint32_t prev = v, next;
  while (cur > (next = p[cur])) {
    p[prev] = next;
    prev = cur;
    cur = next;
  }
  return cur;
}
__device__ __forceinline__ void ts_union(volatile uint32_t *p, uint32_t a, uint32_t b) {
  uint32_t ra = ts_find(p, a), rb = ts_find(p, b);
  while (ra != rb) {
    if (ra < rb) {
      uint32_t t = ra;
      ra = rb;
      rb = t;
    }
    uint32_t old = atomicCAS((uint32_t *)(p + ra), ra, rb);
    if (old == ra) return;
    ra = ts_find(p, old);
    rb = ts_find(p, rb);
  }
}

// The tile kernel: 32-bit offsets inside the tile, a plain per-thread edge
// loop, tile-crossing edges staged in shared memory (flushed with one global
// atomic per tile) with their near endpoint replaced by its tile-local root,
// and the tile-local roots listed for the final roots-only compression.
constexpr int kCutStage = 2048;  // staged cut edges per tile (16 KB)

constexpr int kRootStage = 2048;

template <class T, bool PART>
__global__ void __launch_bounds__(1024)
    k_tile2(uint64_t n, uint64_t m, uint64_t v_begin, uint64_t v_end,
            const uint64_t *__restrict__ rp, const T *__restrict__ col,
            uint32_t *__restrict__ p, PartMap pm, uint32_t tile, uint32_t hub_degree,
            uint32_t *__restrict__ hubs, uint64_t hub_cap, unsigned int *__restrict__ nhubs,
            uint2 *__restrict__ cut, uint64_t cut_cap, unsigned long long *__restrict__ ncut,
            uint32_t *__restrict__ roots, unsigned long long *__restrict__ nroots, int *err) {
  extern __shared__ uint32_t tile_parent[];
  __shared__ uint2 cstage[kCutStage];
  __shared__ uint32_t rstage[kRootStage];
  __shared__ unsigned int ccount, rcount;
  __shared__ unsigned long long cbase, rbase;
  volatile uint32_t *s = tile_parent;
  for (uint64_t t0 = v_begin + (uint64_t)blockIdx.x * tile; t0 < v_end;
       t0 += (uint64_t)gridDim.x * tile) {
    const uint32_t len = (uint32_t)min((uint64_t)tile, v_end - t0);
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) s[i] = i;
    if (threadIdx.x == 0) {
      ccount = 0;
      rcount = 0;
    }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    const uint32_t span = (len + blockDim.x - 1) / blockDim.x * blockDim.x;  // warp-uniform
    for (uint32_t i = threadIdx.x; i < span; i += blockDim.x) {
      const uint64_t v = t0 + i;
      uint64_t b = 0;
      uint32_t deg = 0, lo = 0;
      if (i < len) {
        const uint64_t rb = __ldg(rp + v), re = __ldg(rp + v + 1);
        if (re < rb || re > m) {
          set_err(err, kErrBadOffsets);
        } else if (re - rb > hub_degree) {
          uint32_t slot = atomicAdd(nhubs, 1u);
          if (slot < hub_cap) hubs[slot] = (uint32_t)v;
          else set_err(err, kErrOverflow);
        } else {
          b = rb;
          deg = (uint32_t)(re - rb);
          if (PART) lo = part_lo(pm, (uint32_t)v);
        }
      }
      // every lane walks the warp's longest row so the ballots below see the
      // whole warp (rows above hub_degree were queued instead)
      const uint32_t maxdeg = __reduce_max_sync(0xffffffffu, deg);
      const uint32_t vv = (uint32_t)v, tt = (uint32_t)t0;
      for (uint32_t j = 0; j < maxdeg; ++j) {
        bool emit = false;
        uint32_t u = 0;
        if (j < deg) {
          const uint64_t uu = (uint64_t)__ldg(col + b + j);
          if (uu >= n) {
            set_err(err, kErrBadId);
          } else if ((uint32_t)uu < vv && (!PART || (uint32_t)uu >= lo)) {
            u = (uint32_t)uu;
            if (u >= tt) ts_union(s, i, u - tt);
            else emit = true;  // each undirected edge once, from its larger end
          }
        }
        const unsigned msk = __ballot_sync(0xffffffffu, emit);
        if (msk) {
          const int leader = __ffs(msk) - 1;
          unsigned int base = 0;
          if ((int)lane == leader) base = atomicAdd(&ccount, (unsigned)__popc(msk));
          base = __shfl_sync(0xffffffffu, base, leader);
          if (emit) {
            const unsigned int slot = base + __popc(msk & ((1u << lane) - 1u));
            if (slot < kCutStage) {
              cstage[slot] = make_uint2(i, u);  // near end as a tile index for now
            } else {
              unsigned long long g = atomicAdd(ncut, 1ull);
              if (g < cut_cap) cut[g] = make_uint2(vv, u);
              else set_err(err, kErrOverflow);
            }
          }
        }
      }
    }
    __syncthreads();
    // every vertex stores the global id of its tile-local root; roots are listed
    for (uint32_t i = threadIdx.x; i < span; i += blockDim.x) {
      bool is_root = false;
      if (i < len) {
        uint32_t r = i, nx;
        while ((nx = s[r]) != r) r = nx;
        p[t0 + i] = (uint32_t)(t0 + r);
        is_root = r == i;
      }
      const unsigned msk = __ballot_sync(0xffffffffu, is_root);
      if (msk) {
        const int leader = __ffs(msk) - 1;
        unsigned int base = 0;
        if ((int)lane == leader) base = atomicAdd(&rcount, (unsigned)__popc(msk));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (is_root) {
          const unsigned int slot = base + __popc(msk & ((1u << lane) - 1u));
          if (slot < kRootStage) {
            rstage[slot] = (uint32_t)(t0 + i);
          } else {
            unsigned long long g = atomicAdd(nroots, 1ull);
            roots[g] = (uint32_t)(t0 + i);  // at most n roots: the list holds n
          }
        }
      }
    }
    __syncthreads();
    const unsigned int nc = min(ccount, (unsigned int)kCutStage);
    const unsigned int nr = min(rcount, (unsigned int)kRootStage);
    if (threadIdx.x == 0) {
      cbase = nc ? atomicAdd(ncut, (unsigned long long)nc) : 0ull;
      rbase = nr ? atomicAdd(nroots, (unsigned long long)nr) : 0ull;
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < nc; k += blockDim.x) {
      uint2 c = cstage[k];
      uint32_t r = c.x, nx;
      while ((nx = s[r]) != r) r = nx;  // near end -> its tile-local root
      unsigned long long g = cbase + k;
      if (g < cut_cap) cut[g] = make_uint2((uint32_t)(t0 + r), c.y);
      else set_err(err, kErrOverflow);
    }
    for (uint32_t k = threadIdx.x; k < nr; k += blockDim.x) roots[rbase + k] = rstage[k];
    __syncthreads();
  }
}

// Roots-only compression: every tile-local root points at its final root.
__global__ void k_roots_compress(const uint32_t *__restrict__ roots,
                                 const unsigned long long *__restrict__ nroots, uint32_t *p) {
  const uint64_t cnt = *nroots;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t v = roots[i];
    uint32_t r = ld_cg(p + v), nx;
    if (r == v) continue;
    while ((nx = ld_cg(p + r)) != r) r = nx;
    st_cg(p + v, r);
  }
}

// Every vertex points at a tile-local root (or at a final root): two hops.
__global__ void k_two_hop(uint64_t n, uint32_t *p) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t a = p[v];
    const uint32_t r = ld_cg(p + a);
    if (r != a) p[v] = r;
  }
}

// Edges between tiles, on the global parent array of tile-local roots.
__global__ void k_cut_union(const uint2 *__restrict__ cut, const unsigned long long *__restrict__ ncut,
                            uint64_t cut_cap, uint32_t *p) {
  uint64_t cnt = *ncut;
  if (cnt > cut_cap) cnt = cut_cap;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint2 e = cut[i];
    uf_union(p, e.x, e.y);
  }
}

// Hub rows of the tiled pass: one warp per row, every edge (no first-edge link
// was made for them).
template <class T, bool PART>
__global__ void k_tile_hubs(uint64_t n, const uint64_t *__restrict__ rp, const T *__restrict__ col,
                            uint32_t *p, PartMap pm, const uint32_t *__restrict__ hubs,
                            uint64_t hub_cap, const unsigned int *__restrict__ nhubs, int *err) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t nh = *nhubs;
  if (nh > hub_cap) nh = hub_cap;
  for (uint64_t h = warp; h < nh; h += nwarps) {
    uint32_t v = hubs[h];
    uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);  // checked by k_tile
    uint32_t lo = PART ? part_lo(pm, v) : 0u;
    for (uint64_t k = b + lane; k < e; k += 32) {
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        continue;
      }
      if (u < v && (!PART || (uint32_t)u >= lo)) uf_union(p, v, (uint32_t)u);
    }
  }
}

// Share of sampled edges (u < v, same rank) that leave their tile.
template <class T, bool PART>
__global__ void k_cut_sample(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                             const T *__restrict__ col, PartMap pm, uint32_t tile,
                             uint32_t samples, unsigned long long *__restrict__ counts) {
  unsigned long long tot = 0, cross = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < samples; i += gridDim.x * blockDim.x) {
    uint64_t v = (uint64_t)i * n / samples;
    uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    if (e < b || e > m) continue;
    if (e - b > 64) e = b + 64;
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
}

template <class OUT>
__global__ void k_widen(const uint32_t *__restrict__ in, OUT *__restrict__ out, uint64_t n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    out[v] = (OUT)in[v];
}

// uint32 copy of the ids with the same checks as the hook kernels; a bad id
// becomes the row's own vertex (a self-loop, ignored by every kernel).
template <class T>
__global__ void k_sanitize(uint64_t n, uint64_t m, const uint64_t *__restrict__ rp,
                           const T *__restrict__ col, uint32_t *__restrict__ out, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    Row r;
    if (!load_row(rp, v, m, err, r)) continue;
    for (uint64_t k = r.b; k < r.e; ++k) {
      uint64_t u = (uint64_t)__ldg(col + k);
      if (u >= n) {
        set_err(err, kErrBadId);
        u = v;
      }
      out[k] = (uint32_t)u;
    }
  }
}

template <class T, bool PART>
void run_uf(const Csr &g, uint32_t *parent, const PartMap &pm, uint32_t hub_degree,
            cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  const T *col = static_cast<const T *>(g.col);
  unsigned grid = grid_for(g.n, kBlock, kSMs * 32);
  const uint64_t si = (uint64_t)g.idb;
  cudaEvent_t t0 = c.tic(s);
  k_init<T, PART><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_init", t0, 8 * (g.n + 1) + g.n * si + 4 * g.n);
  const uint64_t hub_cap = g.m / (hub_degree + 1) + 1;
  DevBuf hubs(sizeof(uint32_t) * hub_cap, s, pool);
  DevBuf nh(sizeof(unsigned int), s, pool);
  CCG_CUDA(cudaMemsetAsync(nh.p, 0, sizeof(unsigned int), s));
  // hook: offsets, every id once, one parent gather per edge, own parent r/w
  const uint64_t hook_bytes = 8 * (g.n + 1) + g.m * si + g.m * 4 + 2 * g.n * 4;
  cudaEvent_t t1 = c.tic(s);
  k_hook<T, PART><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, hub_degree,
                                         hubs.as<uint32_t>(), hub_cap, nh.as<unsigned int>(),
                                         g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_hook", t1, hook_bytes);
  cudaEvent_t t2 = c.tic(s);
  k_hook_hubs<T, PART><<<kSMs * 8, kBlock, 0, s>>>(g.n, g.rp, col, parent, pm,
                                                   hubs.as<uint32_t>(), hub_cap,
                                                   nh.as<unsigned int>(), g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_hook_hubs", t2, 0);
  cudaEvent_t t3 = c.tic(s);
  k_compress<<<grid, kBlock, 0, s>>>(g.n, parent);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_compress", t3, 3 * g.n * 4);
  c.add(4, (8 * (g.n + 1) + g.n * si + 4 * g.n) + hook_bytes + 3 * g.n * 4);
}

template <class T, bool PART>
void run_uf_tiled(const Csr &g, uint32_t *parent, const PartMap &pm, const UfTuning &tu,
                  cudaStream_t s, cudaMemPool_t pool, Counters &c, const HostSource *hs) {
  const T *col = static_cast<const T *>(g.col);
  const uint64_t si = (uint64_t)g.idb;
  const uint32_t tile = tu.tile_vertices;
  const int threads = (int)tu.tile_threads;
  const size_t smem = 4ull * tile;  // dynamic: the tile's parent array
  const void *fn = (const void *)k_tile2<T, PART>;
  CCG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  if (per_sm < 1) throw Error(CC_ERR_INVALID, "tile does not fit in shared memory");
  const uint64_t tiles = (g.n + tile - 1) / tile;
  const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)per_sm * kSMs);
  const uint64_t hub_cap = g.m / (tu.hub_degree + 1) + 1;
  const uint64_t cut_cap = g.m + 1;
  DevBuf hubs(4 * hub_cap, s, pool), nh(4, s, pool), cut(8 * cut_cap, s, pool), cnt(16, s, pool);
  DevBuf roots(4 * g.n, s, pool);
  CCG_CUDA(cudaMemsetAsync(nh.p, 0, 4, s));
  CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 16, s));
  unsigned long long *ncut = cnt.as<unsigned long long>(), *nroots = ncut + 1;
  // tile pass: offsets, every id once, own parent written once (the parent
  // chains stay in shared memory); cut edges and roots are counted where read
  const uint64_t tile_bytes = 8 * (g.n + 1) + g.m * si + 4 * g.n;
  cudaEvent_t t0 = c.tic(s);
  if (!hs) {
    k_tile2<T, PART><<<grid, threads, smem, s>>>(g.n, g.m, 0, g.n, g.rp, col, parent, pm, tile,
                                                 tu.hub_degree, hubs.as<uint32_t>(), hub_cap,
                                                 nh.as<unsigned int>(), cut.as<uint2>(), cut_cap,
                                                 ncut, roots.as<uint32_t>(), nroots, g.err);
    CCG_LAUNCH_CHECK();
  } else {
    // Copy tile-aligned chunks of the caller's host CSR on the copy stream and
    // run each chunk's tiles as soon as its slice is on the device: the tile
    // pass overlaps the host-to-device transfer.
    const uint64_t chunk = (uint64_t)grid * tile;  // one full wave of CTAs
    for (uint64_t v0 = 0; v0 < g.n; v0 += chunk) {
      const uint64_t v1 = std::min<uint64_t>(g.n, v0 + chunk);
      const uint64_t e0 = hs->rp[v0], e1 = hs->rp[v1];
      if (e1 < e0 || e1 > g.m) throw Error(CC_ERR_INVALID, "CSR offsets are not monotone or exceed m_dir");
      CCG_CUDA(cudaMemcpyAsync(const_cast<uint64_t *>(g.rp) + v0, hs->rp + v0, 8 * (v1 - v0 + 1),
                               cudaMemcpyHostToDevice, hs->copy));
      if (e1 > e0)
        CCG_CUDA(cudaMemcpyAsync(static_cast<char *>(const_cast<void *>(g.col)) + si * e0,
                                 static_cast<const char *>(hs->col) + si * e0, si * (e1 - e0),
                                 cudaMemcpyHostToDevice, hs->copy));
      cudaEvent_t ev;
      CCG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      CCG_CUDA(cudaEventRecord(ev, hs->copy));
      CCG_CUDA(cudaStreamWaitEvent(s, ev, 0));
      cudaEventDestroy(ev);
      const unsigned cgrid = (unsigned)std::min<uint64_t>((v1 - v0 + tile - 1) / tile, grid);
      k_tile2<T, PART><<<cgrid, threads, smem, s>>>(g.n, g.m, v0, v1, g.rp, col, parent, pm, tile,
                                                    tu.hub_degree, hubs.as<uint32_t>(), hub_cap,
                                                    nh.as<unsigned int>(), cut.as<uint2>(),
                                                    cut_cap, ncut, roots.as<uint32_t>(), nroots,
                                                    g.err);
      CCG_LAUNCH_CHECK();
    }
  }
  c.toc(s, hs ? "uf_tile_streamed" : "uf_tile", t0, tile_bytes);
  cudaEvent_t t1 = c.tic(s);
  k_cut_union<<<kSMs * 16, kBlock, 0, s>>>(cut.as<uint2>(), ncut, cut_cap, parent);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_cut_union", t1, 0);
  cudaEvent_t t2 = c.tic(s);
  k_tile_hubs<T, PART><<<kSMs * 8, kBlock, 0, s>>>(g.n, g.rp, col, parent, pm, hubs.as<uint32_t>(),
                                                   hub_cap, nh.as<unsigned int>(), g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_hook_hubs", t2, 0);
  cudaEvent_t t3 = c.tic(s);
  k_roots_compress<<<kSMs * 16, kBlock, 0, s>>>(roots.as<uint32_t>(), nroots, parent);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_roots_compress", t3, 0);
  cudaEvent_t t4 = c.tic(s);
  k_two_hop<<<grid_for(g.n, kBlock, kSMs * 32), kBlock, 0, s>>>(g.n, parent);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_two_hop", t4, 3 * g.n * 4);
  c.add(5, tile_bytes + 3 * g.n * 4);
}

// Share of tile-crossing edges on a sample of 8192 rows (one small readback).
template <class T, bool PART>
double cut_share(const Csr &g, const PartMap &pm, uint32_t tile, cudaStream_t s,
                 cudaMemPool_t pool, Counters &c) {
  DevBuf cnt(16, s, pool);
  CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 16, s));
  const uint32_t samples = (uint32_t)std::min<uint64_t>(g.n, 8192);
  k_cut_sample<T, PART><<<(samples + 255) / 256, 256, 0, s>>>(
      g.n, g.m, g.rp, static_cast<const T *>(g.col), pm, tile, samples,
      cnt.as<unsigned long long>());
  CCG_LAUNCH_CHECK();
  unsigned long long h[2] = {0, 0};
  CCG_CUDA(cudaMemcpyAsync(h, cnt.p, 16, cudaMemcpyDeviceToHost, s));
  CCG_CUDA(cudaStreamSynchronize(s));
  c.add(1, 0);
  return h[0] ? (double)h[1] / (double)h[0] : 0.0;
}

template <class T, bool PART>
void run_uf_afforest(const Csr &g, uint32_t *parent, const PartMap &pm, uint32_t hub_degree,
                     cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  const T *col = static_cast<const T *>(g.col);
  const uint64_t si = (uint64_t)g.idb;
  const unsigned grid = grid_for(g.n, kBlock, kSMs * 32);
  k_iota_parent<<<grid, kBlock, 0, s>>>(g.n, parent);
  CCG_LAUNCH_CHECK();
  // each link round: offsets, one id, one union (two parent gathers)
  const uint64_t link_bytes = 8 * (g.n + 1) + g.n * si + 2 * g.n * 4;
  for (uint32_t r = 0; r < kAffRounds; ++r) {
    cudaEvent_t t0 = c.tic(s);
    k_aff_link<T, PART><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, r, g.err);
    CCG_LAUNCH_CHECK();
    c.toc(s, "uf_sample_link", t0, link_bytes);
  }
  k_compress<<<grid, kBlock, 0, s>>>(g.n, parent);
  CCG_LAUNCH_CHECK();
  // most frequent root of a sample = the giant component, if there is one
  const uint32_t samples = (uint32_t)std::min<uint64_t>(g.n, 1024);
  DevBuf smp(4 * samples, s, pool);
  k_aff_sample<<<(samples + 255) / 256, 256, 0, s>>>(g.n, parent, samples, 0x5eedull,
                                                     smp.as<uint32_t>());
  CCG_LAUNCH_CHECK();
  std::vector<uint32_t> h(samples);
  CCG_CUDA(cudaMemcpyAsync(h.data(), smp.p, 4 * samples, cudaMemcpyDeviceToHost, s));
  CCG_CUDA(cudaStreamSynchronize(s));
  std::sort(h.begin(), h.end());
  uint32_t L = h.empty() ? kNone : h[0];
  size_t best = 0;
  for (size_t i = 0; i < h.size();) {
    size_t j = i;
    while (j < h.size() && h[j] == h[i]) ++j;
    if (j - i > best) {
      best = j - i;
      L = h[i];
    }
    i = j;
  }
  const uint64_t hub_cap = g.m / (hub_degree + 1) + 1;
  DevBuf hubs(4 * hub_cap, s, pool), nh(4, s, pool);
  CCG_CUDA(cudaMemsetAsync(nh.p, 0, 4, s));
  // remaining pass: offsets, own root, and the ids + unions of the rows
  // outside the giant component (counted as the full edge stream)
  const uint64_t rest_bytes = 8 * (g.n + 1) + g.m * si + g.m * 4 + 2 * g.n * 4;
  cudaEvent_t t1 = c.tic(s);
  k_aff_rest<T, PART><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp, col, parent, pm, L, hub_degree,
                                              hubs.as<uint32_t>(), hub_cap, nh.as<unsigned int>(),
                                              g.err);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_sample_rest", t1, rest_bytes);
  k_aff_rest_hubs<T, PART><<<kSMs * 8, kBlock, 0, s>>>(g.n, g.rp, col, parent, pm,
                                                       hubs.as<uint32_t>(), hub_cap,
                                                       nh.as<unsigned int>(), g.err);
  CCG_LAUNCH_CHECK();
  cudaEvent_t t2 = c.tic(s);
  k_compress<<<grid, kBlock, 0, s>>>(g.n, parent);
  CCG_LAUNCH_CHECK();
  c.toc(s, "uf_compress", t2, 3 * g.n * 4);
  c.add(8, 4 * g.n + kAffRounds * link_bytes + rest_bytes + 6 * g.n * 4);
}

template <class T, bool PART>
void run_uf_mode(const Csr &g, uint32_t *parent, const PartMap &pm, const UfTuning &tu,
                 cudaStream_t s, cudaMemPool_t pool, Counters &c, const HostSource *hs) {
  if (hs) {  // the caller decided on the host that the tiled pass fits this graph
    run_uf_tiled<T, PART>(g, parent, pm, tu, s, pool, c, hs);
    return;
  }
  int mode = tu.mode;
  if (mode == kUfAuto) {
    // the tiled pass wins when most edges stay inside their tile (grids,
    // geometric and angularly ordered graphs); otherwise sampled linking
    mode = (g.n >= 4ull * tu.tile_vertices &&
            cut_share<T, PART>(g, pm, tu.tile_vertices, s, pool, c) < 0.5)
               ? kUfTiled
               : kUfSampled;
  }
  if (mode == kUfTiled) run_uf_tiled<T, PART>(g, parent, pm, tu, s, pool, c, nullptr);
  else if (mode == kUfSampled) run_uf_afforest<T, PART>(g, parent, pm, tu.hub_degree, s, pool, c);
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

double host_cut_share(const uint64_t *rp, const void *col, int idb, uint64_t n, uint64_t m,
                      uint32_t tile) {
  const uint64_t samples = std::min<uint64_t>(n, 8192);
  uint64_t tot = 0, cross = 0;
  for (uint64_t i = 0; i < samples; ++i) {
    const uint64_t v = i * n / samples, t0 = v / tile * tile;
    const uint64_t b = rp[v], e = rp[v + 1];
    if (e < b || e > m) continue;  // malformed rows are reported by the kernels
    for (uint64_t k = b; k < e && k < b + 64; ++k) {
      const uint64_t u = idb == 8 ? static_cast<const uint64_t *>(col)[k]
                                  : static_cast<const uint32_t *>(col)[k];
      if (u >= v) continue;
      ++tot;
      cross += u < t0;
    }
  }
  return tot ? (double)cross / (double)tot : 0.0;
}

void widen_labels(const uint32_t *in, void *out, int out_bytes, uint64_t n, cudaStream_t s,
                  Counters &c) {
  if (n == 0) return;
  unsigned grid = grid_for(n, kBlock, kSMs * 32);
  if (out_bytes == 8)
    k_widen<uint64_t><<<grid, kBlock, 0, s>>>(in, static_cast<uint64_t *>(out), n);
  else
    k_widen<uint32_t><<<grid, kBlock, 0, s>>>(in, static_cast<uint32_t *>(out), n);
  CCG_LAUNCH_CHECK();
  c.add(1, n * 4 + n * (uint64_t)out_bytes);
}

void sanitize_ids(const Csr &g, uint32_t *col32, cudaStream_t s, Counters &c) {
  if (g.n == 0) return;
  unsigned grid = grid_for(g.n, kBlock, kSMs * 32);
  if (g.idb == 8)
    k_sanitize<uint64_t><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp,
                                                 static_cast<const uint64_t *>(g.col), col32, g.err);
  else
    k_sanitize<uint32_t><<<grid, kBlock, 0, s>>>(g.n, g.m, g.rp,
                                                 static_cast<const uint32_t *>(g.col), col32, g.err);
  CCG_LAUNCH_CHECK();
  c.add(1, 8 * (g.n + 1) + g.m * ((uint64_t)g.idb + 4));
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
// Set-up: the first call on a device looks up the device address of the
// scratch array (cudaGetSymbolAddress) with that device current; make that
// first call before any stream capture that should contain this solve.
// ============================================================================
#include <algorithm>
#include <mutex>

namespace {

constexpr uint32_t kNoAllocWords = 1u << 20;                  // 4 MiB
constexpr uint32_t kNoAllocHeader = 64;                       // counter, error word, padding
constexpr uint32_t kNoAllocHubCap = kNoAllocWords - kNoAllocHeader;
constexpr uint32_t kNoAllocHubDegree = 32;

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
  const unsigned grid = grid_for(n, kBlock, kSMs * 32);
  k_init<uint32_t, false><<<grid, kBlock, 0, s>>>(n, m_dir, row_ptr, col, labels_out, pm, err);
  k_hook<uint32_t, false><<<grid, kBlock, 0, s>>>(n, m_dir, row_ptr, col, labels_out, pm,
                                                  kNoAllocHubDegree, hubs, kNoAllocHubCap, nhubs,
                                                  err);
  k_hook_hubs<uint32_t, false><<<kSMs * 8, kBlock, 0, s>>>(n, row_ptr, col, labels_out, pm, hubs,
                                                           kNoAllocHubCap, nhubs, err);
  k_compress<<<grid, kBlock, 0, s>>>(n, labels_out);
  if (cudaGetLastError() != cudaSuccess) return CC_ERR_CUDA;
  int host_err = 0;
  if (cudaMemcpyAsync(&host_err, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return CC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return CC_ERR_CUDA;
  return host_err ? CC_ERR_INVALID : CC_OK;
}

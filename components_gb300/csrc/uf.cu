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

}  // namespace

void uf_components(const Csr &g, uint32_t *parent, const PartMap *pm, uint32_t hub_degree,
                   cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  if (g.n == 0) return;
  if (hub_degree < 1) hub_degree = 1;
  PartMap p = pm ? *pm : PartMap(g.n, 1);
  bool part = pm != nullptr && !(pm->rm == 0 && pm->q == g.n);
  if (g.idb == 8) {
    if (part) run_uf<uint64_t, true>(g, parent, p, hub_degree, s, pool, c);
    else run_uf<uint64_t, false>(g, parent, p, hub_degree, s, pool, c);
  } else {
    if (part) run_uf<uint32_t, true>(g, parent, p, hub_degree, s, pool, c);
    else run_uf<uint32_t, false>(g, parent, p, hub_degree, s, pool, c);
  }
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

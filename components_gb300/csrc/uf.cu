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

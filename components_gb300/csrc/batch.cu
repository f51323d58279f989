// batch.cu - thousands of independent graphs in one solve.
//
// No counterpart in the reference (one graph per driver run).  Each graph is
// solved as the reference's one-rank exp_contraction / all_reduce would: its
// canonical labels are the minimum local id per component.  Layout: one
// segmented CSR (global row offsets, LOCAL neighbour ids) plus vertex offsets.
//
// Schedule, per size bucket (cc_batch_tuning):
//   buckets 0..3  graphs with n <= smem_max_n[b]: one CTA per graph, taken from
//                 a work queue by persistent CTAs; union-find on a parent
//                 array in shared memory; threads stride over vertices
//                 (vertex-parallel) or over edges with a binary search for the
//                 source row (edge-parallel)
//   large         the rest: grid-wide sampled linking on a global parent
//                 array (first two neighbours, a giant root per graph, then
//                 only the rows outside it), hub rows one warp per row
// The launches of one solve are recorded once into a CUDA graph and replayed
// when the same batch and schedule come back.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/cc_batch.h"
#include "kernels.h"

namespace ccg {
namespace {

struct BatchArgs {
  const uint64_t *voff;
  const uint64_t *rp;
  const uint32_t *col;
  uint64_t total_m;
  uint32_t *labels;
  int *err;
};

// One CTA per graph from the bucket's list; persistent CTAs pull work items.
template <bool EDGE_PAR>
__global__ void k_batch_smem(BatchArgs a, const uint32_t *__restrict__ list, uint32_t count,
                             unsigned int *__restrict__ queue) {
  extern __shared__ uint32_t sp[];
  __shared__ uint32_t item;
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(queue, 1u);
    __syncthreads();
    const uint32_t it = item;
    __syncthreads();
    if (it >= count) return;
    const uint32_t gi = list[it];
    const uint64_t v0 = a.voff[gi];
    const uint32_t n = (uint32_t)(a.voff[gi + 1] - v0);
    const uint64_t E0 = a.rp[v0], E1 = a.rp[v0 + n];
    volatile uint32_t *p = sp;
    for (uint32_t v = threadIdx.x; v < n; v += blockDim.x) p[v] = v;
    __syncthreads();
    if (E1 < E0 || E1 > a.total_m) {
      if (threadIdx.x == 0) set_err(a.err, kErrBadOffsets);
    } else if (!EDGE_PAR) {
      for (uint32_t v = threadIdx.x; v < n; v += blockDim.x) {
        uint64_t b = a.rp[v0 + v], e = a.rp[v0 + v + 1];
        if (b < E0 || e > E1 || e < b) {
          set_err(a.err, kErrBadOffsets);
          continue;
        }
        for (uint64_t k = b; k < e; ++k) {
          uint32_t u = __ldg(a.col + k);
          if (u >= n) {
            set_err(a.err, kErrBadId);
            continue;
          }
          if (u < v) smem_union<false>(p, v, u);
        }
      }
    } else {
      const uint64_t *rpg = a.rp + v0;
      for (uint64_t k = E0 + threadIdx.x; k < E1; k += blockDim.x) {
        // source row: last v with rp[v] <= k
        uint32_t lo = 0, hi = n - 1;
        while (lo < hi) {
          uint32_t mid = (lo + hi + 1) >> 1;
          if (__ldg(rpg + mid) <= k) lo = mid;
          else hi = mid - 1;
        }
        uint32_t u = __ldg(a.col + k);
        if (u >= n) {
          set_err(a.err, kErrBadId);
          continue;
        }
        if (u < lo) smem_union<false>(p, lo, u);
      }
    }
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < n; v += blockDim.x) {
      uint32_t r = v, nx;
      while ((nx = p[r]) != r) r = nx;
      a.labels[v0 + v] = r;
    }
    __syncthreads();
  }
}

// ---- grid-wide path for large graphs ----------------------------------------
// Work items are chunks of 1024 vertices: (graph, first local vertex).
struct Chunk {
  uint32_t graph;
  uint32_t first;
};
constexpr uint32_t kChunk = 1024;

// Root of v with path halving; the loads go through L1 (a stale entry still
// names an ancestor, and the CAS in g_union checks roots on the L2 copy), so a
// large graph's hot root entry is not one L2 line that every thread reads.
__device__ __forceinline__ uint32_t g_find(uint32_t *p, uint32_t v) {
  uint32_t cur = p[v];
  if (cur == v) return v;
  uint32_t prev = v, next;
  while (cur > (next = p[cur])) {
    st_cg(p + prev, next);
    prev = cur;
    cur = next;
  }
  return cur;
}
__device__ __forceinline__ void g_union(uint32_t *p, uint32_t a, uint32_t b) {
  uint32_t ra = g_find(p, a), rb = g_find(p, b);
  while (ra != rb) {
    if (ra < rb) {
      uint32_t t = ra;
      ra = rb;
      rb = t;
    }
    uint32_t old = atomicCAS(p + ra, ra, rb);
    if (old == ra) return;
    ra = g_find(p, old);
    rb = g_find(p, rb);
  }
}

// Large graphs run sampled linking (Afforest: Sutton, Ben-Nun, Barak, IPDPS
// 2018), as the single-graph solve does on graphs that do not suit the tiled
// pass: every vertex links to its first two neighbours, the parents are
// compressed, each graph's most frequent root in a sample of its vertices is
// taken as its giant component, and only rows outside it process their
// remaining entries (in both directions: an edge between a giant vertex and
// another is processed from the other end).  Ids in the skipped entries are
// never read.  The parent array is indexed by global vertex id (it spans
// total_n entries; only the large graphs' entries are used).
__global__ void k_large_iota(BatchArgs a, const Chunk *__restrict__ chunks, uint32_t nchunks,
                             uint32_t *__restrict__ par) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < (uint64_t)nchunks * kChunk;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const Chunk c = chunks[t / kChunk];
    const uint64_t v0 = a.voff[c.graph];
    const uint32_t n = (uint32_t)(a.voff[c.graph + 1] - v0);
    const uint32_t v = c.first + (uint32_t)(t % kChunk);
    if (v >= n) continue;
    const uint64_t b = a.rp[v0 + v], e = a.rp[v0 + v + 1];
    if (e < b || e > a.total_m) set_err(a.err, kErrBadOffsets);
    par[v0 + v] = (uint32_t)(v0 + v);
  }
}

// Link round r: every vertex with more than r entries unites with its r-th
// neighbour.
__global__ void k_large_link(BatchArgs a, const Chunk *__restrict__ chunks, uint32_t nchunks,
                             uint32_t *par, uint32_t r) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < (uint64_t)nchunks * kChunk;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const Chunk c = chunks[t / kChunk];
    const uint64_t v0 = a.voff[c.graph];
    const uint32_t n = (uint32_t)(a.voff[c.graph + 1] - v0);
    const uint32_t v = c.first + (uint32_t)(t % kChunk);
    if (v >= n) continue;
    const uint64_t b = a.rp[v0 + v], e = a.rp[v0 + v + 1];
    if (e < b || e > a.total_m || e - b <= r) continue;  // bad offsets: reported by k_large_iota
    const uint32_t u = __ldg(a.col + b + r);
    if (u >= n) {
      set_err(a.err, kErrBadId);
      continue;
    }
    g_union(par, (uint32_t)(v0 + v), (uint32_t)(v0 + u));
  }
}

// Every large vertex points at its root (no union runs meanwhile).
__global__ void k_large_compress(BatchArgs a, const Chunk *__restrict__ chunks, uint32_t nchunks,
                                 uint32_t *par) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < (uint64_t)nchunks * kChunk;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const Chunk c = chunks[t / kChunk];
    const uint64_t v0 = a.voff[c.graph];
    const uint32_t n = (uint32_t)(a.voff[c.graph + 1] - v0);
    const uint32_t v = c.first + (uint32_t)(t % kChunk);
    if (v >= n) continue;
    uint32_t r = (uint32_t)(v0 + v), nx;
    while ((nx = par[r]) != r) r = nx;
    if (par[v0 + v] != r) par[v0 + v] = r;
  }
}

// Giant root of each large graph: the most frequent root among kModeSamples
// hashed vertices of the graph (one CTA of kModeSamples threads per graph:
// bitonic sort of the roots in shared memory, then the longest run).
constexpr uint32_t kModeSamples = 256;
__global__ void __launch_bounds__(kModeSamples) k_large_mode(BatchArgs a, const uint32_t *__restrict__ big,
                                                             uint32_t nbig, const uint32_t *par,
                                                             uint32_t *__restrict__ giant) {
  __shared__ uint32_t sm[kModeSamples];
  const uint32_t i = threadIdx.x;
  for (uint32_t bi = blockIdx.x; bi < nbig; bi += gridDim.x) {
    const uint32_t g = big[bi];
    const uint64_t v0 = a.voff[g];
    const uint64_t n = a.voff[g + 1] - v0;
    uint32_t r = (uint32_t)(v0 + mix64(0x5eedull + (uint64_t)g * kModeSamples + i) % n), nx;
    while ((nx = par[r]) != r) r = nx;
    sm[i] = r;
    __syncthreads();
    for (uint32_t k = 2; k <= kModeSamples; k <<= 1) {
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        const uint32_t ixj = i ^ j;
        if (ixj > i) {
          const uint32_t x = sm[i], y = sm[ixj];
          if ((x > y) == ((i & k) == 0)) {
            sm[i] = y;
            sm[ixj] = x;
          }
        }
        __syncthreads();
      }
    }
    if (i == 0) {
      uint32_t best = sm[0], best_len = 1, run = 1;
      for (uint32_t k = 1; k < kModeSamples; ++k) {
        run = sm[k] == sm[k - 1] ? run + 1 : 1;
        if (run > best_len) {
          best_len = run;
          best = sm[k];
        }
      }
      giant[g] = best;
    }
    __syncthreads();
  }
}

// Rows outside their graph's giant root process their remaining entries (the
// first two were linked); rows longer than hub_degree go to k_large_hubs.
__global__ void k_large_rest(BatchArgs a, const Chunk *__restrict__ chunks, uint32_t nchunks,
                             uint32_t *par, const uint32_t *__restrict__ giant, uint32_t hub_degree,
                             uint32_t *__restrict__ hubs, uint64_t hub_cap,
                             unsigned int *__restrict__ nh) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < (uint64_t)nchunks * kChunk;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const Chunk c = chunks[t / kChunk];
    const uint64_t v0 = a.voff[c.graph];
    const uint32_t n = (uint32_t)(a.voff[c.graph + 1] - v0);
    const uint32_t v = c.first + (uint32_t)(t % kChunk);
    if (v >= n) continue;
    // compressed before this pass: a vertex that held the giant root then is
    // in the giant component for good (a later walk may move it to an
    // ancestor; such a row is then processed, which is only more work)
    if (ld_cg(par + v0 + v) == giant[c.graph]) continue;
    const uint64_t b = a.rp[v0 + v], e = a.rp[v0 + v + 1];
    if (e < b || e > a.total_m || e - b <= 2) continue;
    if (e - b > hub_degree) {
      const uint32_t slot = atomicAdd(nh, 1u);
      if (slot < hub_cap) hubs[slot] = (uint32_t)(v0 + v);
      else set_err(a.err, kErrOverflow);
      continue;
    }
    for (uint64_t k = b + 2; k < e; ++k) {
      const uint32_t u = __ldg(a.col + k);
      if (u >= n) {
        set_err(a.err, kErrBadId);
        continue;
      }
      g_union(par, (uint32_t)(v0 + v), (uint32_t)(v0 + u));
    }
  }
}

// Hub rows outside the giant component: one warp per row, every entry after
// the two linked ones.  The graph of a hub is found by binary search over the
// vertex offsets of the large graphs.
__global__ void k_large_hubs(BatchArgs a, const uint32_t *__restrict__ big, uint32_t nbig,
                             uint32_t *par, const uint32_t *__restrict__ hubs, uint64_t hub_cap,
                             const unsigned int *__restrict__ nh) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t cnt = *nh;
  if (cnt > hub_cap) cnt = hub_cap;
  for (uint64_t h = warp; h < cnt; h += nwarps) {
    uint32_t gv = hubs[h];
    uint32_t lo = 0, hi = nbig - 1;  // last large graph with voff <= gv
    while (lo < hi) {
      uint32_t mid = (lo + hi + 1) >> 1;
      if (a.voff[big[mid]] <= gv) lo = mid;
      else hi = mid - 1;
    }
    uint32_t gi = big[lo];
    uint64_t v0 = a.voff[gi];
    uint32_t n = (uint32_t)(a.voff[gi + 1] - v0);
    uint64_t b = a.rp[gv], e = a.rp[gv + 1];
    for (uint64_t k = b + 2 + lane; k < e; k += 32) {
      uint32_t u = __ldg(a.col + k);
      if (u >= n) {
        set_err(a.err, kErrBadId);
        continue;
      }
      g_union(par, gv, (uint32_t)(v0 + u));
    }
  }
}

__global__ void k_large_finish(BatchArgs a, const Chunk *__restrict__ chunks, uint32_t nchunks,
                               const uint32_t *par) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < (uint64_t)nchunks * kChunk;
       t += (uint64_t)gridDim.x * blockDim.x) {
    Chunk c = chunks[t / kChunk];
    uint64_t v0 = a.voff[c.graph];
    uint32_t n = (uint32_t)(a.voff[c.graph + 1] - v0);
    uint32_t v = c.first + (uint32_t)(t % kChunk);
    if (v >= n) continue;
    uint32_t r = (uint32_t)(v0 + v), nx;
    while ((nx = par[r]) != r) r = nx;  // roots are final here: L1 reads are safe
    a.labels[v0 + v] = (uint32_t)(r - v0);
  }
}

}  // namespace

// ---- host side ---------------------------------------------------------------

struct BatchPlan {
  std::vector<uint32_t> lists[CC_BATCH_BUCKETS];
  std::vector<uint32_t> big;
  std::vector<Chunk> chunks;
  uint32_t bucket_n[CC_BATCH_BUCKETS] = {0, 0, 0, 0};
};

BatchPlan plan_batch(const std::vector<uint64_t> &voff, const cc_batch_tuning &t) {
  BatchPlan P;
  const uint32_t k = (uint32_t)voff.size() - 1;
  for (uint32_t i = 0; i < k; ++i) {
    uint64_t n = voff[i + 1] - voff[i];
    int b = 0;
    while (b < CC_BATCH_BUCKETS && (t.smem_max_n[b] == 0 || n > t.smem_max_n[b])) ++b;
    if (b < CC_BATCH_BUCKETS && n > 0) {
      P.lists[b].push_back(i);
    } else if (n > 0) {
      P.big.push_back(i);
      for (uint64_t f = 0; f < n; f += kChunk) P.chunks.push_back({i, (uint32_t)f});
    }
  }
  for (int b = 0; b < CC_BATCH_BUCKETS; ++b) P.bucket_n[b] = t.smem_max_n[b];
  return P;
}

struct BatchDev {
  DevBuf lists[CC_BATCH_BUCKETS], big, chunks, queues, par, hubs, nh, giant;
  uint64_t hub_cap = 0;
};

void upload_plan(const BatchPlan &P, uint64_t total_n, uint64_t total_m, uint32_t hub_degree,
                 BatchDev &D, cudaStream_t s, cudaMemPool_t pool) {
  for (int b = 0; b < CC_BATCH_BUCKETS; ++b) {
    D.lists[b].alloc(4 * (P.lists[b].size() + 1), s, pool);
    if (!P.lists[b].empty())
      CCG_CUDA(cudaMemcpyAsync(D.lists[b].p, P.lists[b].data(), 4 * P.lists[b].size(),
                               cudaMemcpyHostToDevice, s));
  }
  D.big.alloc(4 * (P.big.size() + 1), s, pool);
  if (!P.big.empty())
    CCG_CUDA(cudaMemcpyAsync(D.big.p, P.big.data(), 4 * P.big.size(), cudaMemcpyHostToDevice, s));
  D.chunks.alloc(sizeof(Chunk) * (P.chunks.size() + 1), s, pool);
  if (!P.chunks.empty())
    CCG_CUDA(cudaMemcpyAsync(D.chunks.p, P.chunks.data(), sizeof(Chunk) * P.chunks.size(),
                             cudaMemcpyHostToDevice, s));
  D.queues.alloc(4 * (CC_BATCH_BUCKETS + 1), s, pool);
  D.par.alloc(4 * (P.chunks.empty() ? 1 : total_n), s, pool);
  // giant root per graph, indexed by graph id (the large graphs' ids ascend in P.big)
  D.giant.alloc(4 * (P.big.empty() ? 1 : (uint64_t)P.big.back() + 1), s, pool);
  D.hub_cap = total_m / (hub_degree + 1) + 1;
  D.hubs.alloc(4 * D.hub_cap, s, pool);
  D.nh.alloc(4, s, pool);
  CCG_CUDA(cudaStreamSynchronize(s));  // host vectors of P may go away
}

static int smem_blocks_per_sm(const void *fn, int threads, size_t smem) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

void launch_batch(const BatchArgs &a, const BatchPlan &P, BatchDev &D, const cc_batch_tuning &t,
                  cudaStream_t s, Counters &c) {
  CCG_CUDA(cudaMemsetAsync(D.queues.p, 0, 4 * (CC_BATCH_BUCKETS + 1), s));
  CCG_CUDA(cudaMemsetAsync(D.nh.p, 0, 4, s));
  for (int b = 0; b < CC_BATCH_BUCKETS; ++b) {
    uint32_t cnt = (uint32_t)P.lists[b].size();
    if (!cnt) continue;
    int threads = (int)(t.threads[b] ? t.threads[b] : 256);
    size_t smem = 4ull * P.bucket_n[b];
    const void *fn = t.edge_parallel[b] ? (const void *)k_batch_smem<true>
                                        : (const void *)k_batch_smem<false>;
    if (smem > 48 * 1024)
      CCG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = smem_blocks_per_sm(fn, threads, smem);
    unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)per_sm * num_sms(), cnt);
    unsigned int *q = D.queues.as<unsigned int>() + b;
    if (t.edge_parallel[b])
      k_batch_smem<true><<<grid, threads, smem, s>>>(a, D.lists[b].as<uint32_t>(), cnt, q);
    else
      k_batch_smem<false><<<grid, threads, smem, s>>>(a, D.lists[b].as<uint32_t>(), cnt, q);
    CCG_LAUNCH_CHECK();
    c.add(1, 0);
  }
  if (!P.chunks.empty()) {
    uint32_t nch = (uint32_t)P.chunks.size();
    unsigned grid = grid_for((uint64_t)nch * kChunk, kBlock, num_sms() * 32);
    uint32_t *par = D.par.as<uint32_t>();
    const Chunk *ch = D.chunks.as<Chunk>();
    const uint32_t nbig = (uint32_t)P.big.size();
    k_large_iota<<<grid, kBlock, 0, s>>>(a, ch, nch, par);
    CCG_LAUNCH_CHECK();
    for (uint32_t r = 0; r < 2; ++r) {
      k_large_link<<<grid, kBlock, 0, s>>>(a, ch, nch, par, r);
      CCG_LAUNCH_CHECK();
    }
    k_large_compress<<<grid, kBlock, 0, s>>>(a, ch, nch, par);
    CCG_LAUNCH_CHECK();
    k_large_mode<<<std::min<uint32_t>(nbig, (uint32_t)num_sms() * 8), kModeSamples, 0, s>>>(
        a, D.big.as<uint32_t>(), nbig, par, D.giant.as<uint32_t>());
    CCG_LAUNCH_CHECK();
    k_large_rest<<<grid, kBlock, 0, s>>>(a, ch, nch, par, D.giant.as<uint32_t>(),
                                         t.hub_degree ? t.hub_degree : 32, D.hubs.as<uint32_t>(),
                                         D.hub_cap, D.nh.as<unsigned int>());
    CCG_LAUNCH_CHECK();
    k_large_hubs<<<num_sms() * 8, kBlock, 0, s>>>(a, D.big.as<uint32_t>(), nbig, par,
                                             D.hubs.as<uint32_t>(), D.hub_cap,
                                             D.nh.as<unsigned int>());
    CCG_LAUNCH_CHECK();
    k_large_finish<<<grid, kBlock, 0, s>>>(a, ch, nch, par);
    CCG_LAUNCH_CHECK();
    c.add(8, 0);
  }
}

}  // namespace ccg

// ============================== C ABI ==========================================
#include "ctx.h"

namespace ccg {

struct BatchCache {
  uint64_t key = 0;
  BatchPlan plan;
  BatchDev dev;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

void batch_cache_free(BatchCache *c) {
  if (!c) return;
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  delete c;
}

namespace {

uint64_t fnv(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 0x100000001b3ull;
  return h;
}

void check_batch(const cc_batch *b) {
  if (!b) throw Error(CC_ERR_INVALID, "batch is NULL");
  if (b->where != CC_HOST && b->where != CC_DEVICE) throw Error(CC_ERR_INVALID, "bad where");
  if (!b->voff) throw Error(CC_ERR_INVALID, "voff is NULL");
  if (b->total_n > 0 && !b->row_ptr) throw Error(CC_ERR_INVALID, "row_ptr is NULL");
  if (b->total_m > 0 && !b->col) throw Error(CC_ERR_INVALID, "col is NULL");
  if (b->total_n >= 0xffffffffull) throw Error(CC_ERR_UNSUPPORTED, "total_n >= 2^32-1");
}

std::vector<uint64_t> host_voff(const cc_batch *b, cudaStream_t s) {
  std::vector<uint64_t> v(b->k + 1);
  if (b->where == CC_HOST) {
    std::memcpy(v.data(), b->voff, 8 * (b->k + 1));
  } else {
    CCG_CUDA(cudaMemcpyAsync(v.data(), b->voff, 8 * (b->k + 1), cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
  }
  if (v[0] != 0 || v[b->k] != b->total_n) throw Error(CC_ERR_INVALID, "voff[0] must be 0 and voff[k] = total_n");
  for (uint32_t i = 0; i < b->k; ++i)
    if (v[i + 1] < v[i]) throw Error(CC_ERR_INVALID, "voff is not monotone");
  return v;
}

// Time `reps` launches of the plan P under tuning t (device batch a).
double time_plan(const BatchArgs &a, const BatchPlan &P, const cc_batch_tuning &t, uint64_t total_n,
                 uint64_t total_m, int reps, cudaStream_t s, cudaMemPool_t pool) {
  BatchDev D;
  upload_plan(P, total_n, total_m, t.hub_degree ? t.hub_degree : 32, D, s, pool);
  Counters c;
  launch_batch(a, P, D, t, s, c);  // warm-up
  cudaEvent_t e0, e1;
  CCG_CUDA(cudaEventCreate(&e0));
  CCG_CUDA(cudaEventCreate(&e1));
  CCG_CUDA(cudaEventRecord(e0, s));
  for (int r = 0; r < reps; ++r) launch_batch(a, P, D, t, s, c);
  CCG_CUDA(cudaEventRecord(e1, s));
  CCG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

// Per-graph row offsets starting at 0 for the plain per-graph loop: graph i's
// n_i + 1 offsets land at local[voff[i] + i ...] (one CTA per graph).
__global__ void k_rebase_offsets(const uint64_t *__restrict__ voff, const uint64_t *__restrict__ rp,
                                 uint32_t k, uint64_t *__restrict__ local) {
  for (uint32_t i = blockIdx.x; i < k; i += gridDim.x) {
    const uint64_t a = voff[i], b = voff[i + 1], base = rp[a];
    for (uint64_t j = threadIdx.x; j <= b - a; j += blockDim.x) local[a + i + j] = rp[a + j] - base;
  }
}

}  // namespace
}  // namespace ccg

extern "C" {

void cc_batch_tuning_default(cc_batch_tuning *t) {
  if (!t) return;
  std::memset(t, 0, sizeof(*t));
  const uint32_t bounds[CC_BATCH_BUCKETS] = {1024, 4096, 16384, 49152};
  for (int b = 0; b < CC_BATCH_BUCKETS; ++b) {
    t->smem_max_n[b] = bounds[b];
    t->threads[b] = b < 2 ? 256 : 512;
    t->edge_parallel[b] = 0;
  }
  t->hub_degree = 32;
  t->use_graph = 1;
}

int cc_batch_run(cc_ctx *ctx, const cc_batch *b, const cc_batch_tuning *tuning, uint32_t *labels_out,
                 uint32_t labels_where) {
  using namespace ccg;
  return guard([&] {
    if (!ctx) throw Error(CC_ERR_INVALID, "context is NULL");
    check_batch(b);
    if (labels_where != CC_HOST && labels_where != CC_DEVICE)
      throw Error(CC_ERR_INVALID, "bad labels_where");
    if (b->total_n > 0 && !labels_out) throw Error(CC_ERR_INVALID, "labels_out is NULL");
    CCG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    cc_batch_tuning t;
    if (tuning) t = *tuning;
    else cc_batch_tuning_default(&t);
    for (int i = 0; i < CC_BATCH_BUCKETS; ++i) {
      if (t.smem_max_n[i] > 56 * 1024) throw Error(CC_ERR_INVALID, "smem_max_n above 56K vertices");
      if (t.threads[i] && (t.threads[i] % 32 || t.threads[i] > 1024))
        throw Error(CC_ERR_INVALID, "threads must be a multiple of 32 up to 1024");
    }
    cc_stats st;
    std::memset(&st, 0, sizeof(st));
    cudaEvent_t ev[4];
    for (auto &e : ev) CCG_CUDA(cudaEventCreate(&e));
    struct EvGuard {
      cudaEvent_t *e;
      ~EvGuard() {
        for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
      }
    } evg{ev};
    CCG_CUDA(cudaEventRecord(ev[0], s));
    std::vector<uint64_t> voff = host_voff(b, s);
    DevBuf voff_d, rp_d, col_d, lab_d;
    BatchArgs a;
    a.total_m = b->total_m;
    a.err = ctx->d_err;
    if (b->where == CC_HOST) {
      voff_d.alloc(8 * (b->k + 1), s, ctx->pool);
      rp_d.alloc(8 * (b->total_n + 1), s, ctx->pool);
      col_d.alloc(4 * (b->total_m ? b->total_m : 1), s, ctx->pool);
      CCG_CUDA(cudaMemcpyAsync(voff_d.p, b->voff, 8 * (b->k + 1), cudaMemcpyHostToDevice, s));
      CCG_CUDA(cudaMemcpyAsync(rp_d.p, b->row_ptr, 8 * (b->total_n + 1), cudaMemcpyHostToDevice, s));
      if (b->total_m)
        CCG_CUDA(cudaMemcpyAsync(col_d.p, b->col, 4 * b->total_m, cudaMemcpyHostToDevice, s));
      st.h2d_bytes = 8 * (b->k + 1) + 8 * (b->total_n + 1) + 4 * b->total_m;
      a.voff = voff_d.as<uint64_t>();
      a.rp = rp_d.as<uint64_t>();
      a.col = col_d.as<uint32_t>();
    } else {
      a.voff = b->voff;
      a.rp = b->row_ptr;
      a.col = b->col;
    }
    if (labels_where == CC_DEVICE) {
      a.labels = labels_out;
    } else {
      lab_d.alloc(4 * (b->total_n ? b->total_n : 1), s, ctx->pool);
      a.labels = lab_d.as<uint32_t>();
    }
    CCG_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), s));
    CCG_CUDA(cudaEventRecord(ev[1], s));
    Counters c;
    uint64_t key = fnv(0xcbf29ce484222325ull, voff.data(), 8 * voff.size());
    const void *ptrs[5] = {a.voff, a.rp, a.col, a.labels, (void *)(uintptr_t)b->total_m};
    key = fnv(key, ptrs, sizeof(ptrs));
    key = fnv(key, &t, sizeof(t));
    BatchCache *cache = ctx->batch;
    if (t.use_graph && cache && cache->key == key && cache->exec) {
      CCG_CUDA(cudaGraphLaunch(cache->exec, s));
      c.add(1, 0);
    } else {
      std::unique_ptr<BatchCache> nc(new BatchCache());
      nc->key = key;
      nc->plan = plan_batch(voff, t);
      upload_plan(nc->plan, b->total_n, b->total_m, t.hub_degree ? t.hub_degree : 32, nc->dev, s,
                  ctx->pool);
      if (t.use_graph && b->where == CC_DEVICE) {
        CCG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
          launch_batch(a, nc->plan, nc->dev, t, s, c);
        } catch (...) {
          cudaGraph_t g = nullptr;
          cudaStreamEndCapture(s, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        CCG_CUDA(cudaStreamEndCapture(s, &nc->graph));
        CCG_CUDA(cudaGraphInstantiate(&nc->exec, nc->graph, 0));
        CCG_CUDA(cudaGraphLaunch(nc->exec, s));
        batch_cache_free(ctx->batch);
        ctx->batch = nc.release();
      } else {
        launch_batch(a, nc->plan, nc->dev, t, s, c);
        CCG_CUDA(cudaStreamSynchronize(s));  // nc's buffers are freed on scope exit
      }
    }
    CCG_CUDA(cudaEventRecord(ev[2], s));
    if (labels_where == CC_HOST && b->total_n) {
      CCG_CUDA(cudaMemcpyAsync(labels_out, a.labels, 4 * b->total_n, cudaMemcpyDeviceToHost, s));
      st.d2h_bytes = 4 * b->total_n;
    }
    CCG_CUDA(cudaEventRecord(ev[3], s));
    CCG_CUDA(cudaStreamSynchronize(s));
    throw_on_kernel_error(ctx, s);
    float t_solve = 0.f, t_total = 0.f;
    cudaEventElapsedTime(&t_solve, ev[1], ev[2]);
    cudaEventElapsedTime(&t_total, ev[0], ev[3]);
    st.solve_ms = t_solve;
    st.total_ms = t_total;
    st.kernel_launches = c.launches;
    // hook-and-compress bytes: offsets, ids, one parent gather per edge, labels
    st.bytes_algorithmic = 8 * (b->total_n + b->k) + 4 * b->total_m * 2 + 3 * 4 * b->total_n;
    ctx->stats = st;
  });
}

int cc_batch_autotune(cc_ctx *ctx, const cc_batch *b, int reps, cc_batch_tuning *out) {
  using namespace ccg;
  return guard([&] {
    if (!ctx || !out) throw Error(CC_ERR_INVALID, "NULL argument");
    check_batch(b);
    if (b->where != CC_DEVICE) throw Error(CC_ERR_INVALID, "autotune takes a device batch");
    if (reps < 1) reps = 1;
    CCG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    std::vector<uint64_t> voff = host_voff(b, s);
    DevBuf lab(4 * (b->total_n ? b->total_n : 1), s, ctx->pool);
    BatchArgs a{b->voff, b->row_ptr, b->col, b->total_m, lab.as<uint32_t>(), ctx->d_err};
    cc_batch_tuning best;
    cc_batch_tuning_default(&best);
    best.use_graph = 0;
    BatchPlan full = plan_batch(voff, best);
    const uint32_t cand_threads[3] = {128, 256, 512};
    // per bucket: CTA size x vertex/edge-parallel
    for (int bk = 0; bk < CC_BATCH_BUCKETS; ++bk) {
      if (full.lists[bk].empty()) continue;
      BatchPlan only;
      only.lists[bk] = full.lists[bk];
      for (int i = 0; i < CC_BATCH_BUCKETS; ++i) only.bucket_n[i] = full.bucket_n[i];
      double best_ms = 1e30;
      for (uint32_t th : cand_threads)
        for (uint32_t ep = 0; ep < 2; ++ep) {
          cc_batch_tuning t = best;
          t.threads[bk] = th;
          t.edge_parallel[bk] = ep;
          double ms = time_plan(a, only, t, b->total_n, b->total_m, reps, s, ctx->pool);
          if (ms < best_ms) {
            best_ms = ms;
            best.threads[bk] = th;
            best.edge_parallel[bk] = ep;
          }
        }
      // the largest bucket competes with the grid-wide path for its graphs
      if (bk == CC_BATCH_BUCKETS - 1) {
        cc_batch_tuning t = best;
        t.smem_max_n[bk] = 0;
        BatchPlan alt = plan_batch(voff, t);
        BatchPlan alt_only;
        alt_only.big = alt.big;
        alt_only.chunks.clear();
        for (uint32_t gi : full.lists[bk]) {
          uint64_t n = voff[gi + 1] - voff[gi];
          for (uint64_t f = 0; f < n; f += kChunk) alt_only.chunks.push_back({gi, (uint32_t)f});
        }
        alt_only.big = full.lists[bk];
        double ms = time_plan(a, alt_only, t, b->total_n, b->total_m, reps, s, ctx->pool);
        if (ms < best_ms) best.smem_max_n[bk] = 0;
      }
    }
    // grid-wide path: hub threshold (vertex- vs edge-parallel rows)
    BatchPlan big = plan_batch(voff, best);
    if (!big.chunks.empty()) {
      BatchPlan only;
      only.big = big.big;
      only.chunks = big.chunks;
      double best_ms = 1e30;
      for (uint32_t hd : {16u, 32u, 64u, 256u}) {
        cc_batch_tuning t = best;
        t.hub_degree = hd;
        double ms = time_plan(a, only, t, b->total_n, b->total_m, reps, s, ctx->pool);
        if (ms < best_ms) {
          best_ms = ms;
          best.hub_degree = hd;
        }
      }
    }
    throw_on_kernel_error(ctx, s);
    best.use_graph = 1;
    *out = best;
  });
}

int cc_batch_run_plain(cc_ctx *ctx, const cc_batch *b, cc_algo algo, const cc_config *cfg,
                       uint64_t seed, uint32_t *labels_out) {
  using namespace ccg;
  if (!ctx) return CC_ERR_INVALID;
  int rc = guard([&] {
    check_batch(b);
    if (b->where != CC_DEVICE) throw Error(CC_ERR_INVALID, "the plain loop takes device arrays");
    if (b->total_n > 0 && !labels_out) throw Error(CC_ERR_INVALID, "labels_out is NULL");
    CCG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const std::vector<uint64_t> voff = host_voff(b, s);
    std::vector<uint64_t> bounds(b->k + 1);  // global row offset at each graph's first row
    for (uint32_t i = 0; i <= b->k; ++i)
      CCG_CUDA(cudaMemcpyAsync(&bounds[i], b->row_ptr + voff[i], 8, cudaMemcpyDeviceToHost, s));
    ctx->plain_rp.alloc(8 * (b->total_n + b->k + 1), s, ctx->pool);
    if (b->k)
      k_rebase_offsets<<<std::min<uint32_t>(b->k, 65535), 256, 0, s>>>(b->voff, b->row_ptr, b->k,
                                                                      ctx->plain_rp.as<uint64_t>());
    CCG_LAUNCH_CHECK();
    CCG_CUDA(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < b->k; ++i) {
      cc_csr g;
      std::memset(&g, 0, sizeof(g));
      g.n = voff[i + 1] - voff[i];
      g.m_dir = bounds[i + 1] - bounds[i];
      g.row_ptr = ctx->plain_rp.as<uint64_t>() + voff[i] + i;
      g.col = b->col + bounds[i];
      g.id_bytes = 4;
      g.num_parts = 1;
      g.where = CC_DEVICE;
      if (g.n == 0) continue;
      const int st = cc_ctx_run(ctx, &g, algo, cfg, seed, labels_out + voff[i], CC_DEVICE);
      if (st != CC_OK) throw Error(st, "plain solve of one graph failed");
    }
  });
  return rc;
}

}  // extern "C"

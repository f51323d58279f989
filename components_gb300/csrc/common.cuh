// common.cuh - shared device helpers of libccgpu (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/cc_gpu.h"

namespace ccg {

// Internal failure: carries a status code up to the C ABI, which converts it
// to an int return.  Nothing below the ABI calls exit().
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &msg) : std::runtime_error(msg), status(s) {}
};

#define CCG_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      int st_ = (e_ == cudaErrorMemoryAllocation) ? CC_ERR_OOM : CC_ERR_CUDA; \
      throw ::ccg::Error(st_, std::string(#call) + " failed: " +              \
                                  cudaGetErrorString(e_) + " at " +           \
                                  __FILE__ + ":" + std::to_string(__LINE__)); \
    }                                                                         \
  } while (0)

#define CCG_LAUNCH_CHECK() CCG_CUDA(cudaGetLastError())

constexpr uint32_t kNone = 0xffffffffu;
constexpr int kBlock = 256;
// SMs of the current device (152 on a GB300: two dies of 76), queried once per
// device; grid caps are multiples of it.
inline int num_sms() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 152;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

// Per-solve launch bookkeeping, reported through cc_stats.  With prof on,
// tic()/toc() bracket single kernels with CUDA events on their stream; the
// durations are read after the solve (cc_stats.kernels).
struct Counters {
  uint64_t launches = 0;
  uint64_t bytes = 0;  // algorithmic bytes (formulas next to each launcher)
  bool prof = false;
  struct Rec {
    const char *name;
    cudaEvent_t a, b;
    uint64_t bytes;
  };
  std::vector<Rec> recs;
  // Events for tic/toc: taken from `pool` (owned by a context and kept across
  // solves, so profiling adds no event creation per solve) or, without one,
  // created and destroyed per use.
  std::vector<cudaEvent_t> *pool = nullptr;
  size_t used = 0;
  void add(uint64_t nl, uint64_t b) {
    launches += nl;
    bytes += b;
  }
  cudaEvent_t event() {
    if (pool) {
      if (used == pool->size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        pool->push_back(e);
      }
      return (*pool)[used++];
    }
    cudaEvent_t e;
    return cudaEventCreate(&e) == cudaSuccess ? e : nullptr;
  }
  cudaEvent_t tic(cudaStream_t s) {
    if (!prof) return nullptr;
    cudaEvent_t e = event();
    if (e) cudaEventRecord(e, s);
    return e;
  }
  void toc(cudaStream_t s, const char *name, cudaEvent_t a, uint64_t b) {
    if (!prof || !a) return;
    cudaEvent_t e = event();
    if (!e) return;
    cudaEventRecord(e, s);
    recs.push_back({name, a, e, b});
  }
  void clear_recs() {
    if (!pool) {
      for (auto &r : recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
      }
    }
    recs.clear();
    used = 0;
  }
};

// Error word written by kernels that read a caller's CSR: a bounds failure
// records its code and the access is skipped (no fault, no trap).
enum : int { kErrNone = 0, kErrBadOffsets = 1, kErrBadId = 2, kErrOverflow = 3 };
__device__ __forceinline__ void set_err(int *err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// Stream-ordered device buffer drawn from the context's memory pool.  The pool
// keeps freed blocks (release threshold = max), so steady-state solves do not
// reach cudaMalloc.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaStream_t s = nullptr;
  cudaMemPool_t pool = nullptr;
  DevBuf() = default;
  DevBuf(size_t nbytes, cudaStream_t st, cudaMemPool_t pl) { alloc(nbytes, st, pl); }
  void alloc(size_t nbytes, cudaStream_t st, cudaMemPool_t pl) {
    release();
    s = st;
    pool = pl;
    bytes = nbytes;
    if (nbytes == 0) return;
    CCG_CUDA(cudaMallocFromPoolAsync(&p, nbytes, pool, s));
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    bytes = 0;
  }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept { *this = std::move(o); }
  DevBuf &operator=(DevBuf &&o) noexcept {
    release();
    p = o.p; bytes = o.bytes; s = o.s; pool = o.pool;
    o.p = nullptr; o.bytes = 0;
    return *this;
  }
  template <class T> T *as() const { return static_cast<T *>(p); }
};

inline unsigned grid_for(uint64_t work, int block = kBlock, unsigned cap = num_sms() * 16) {
  uint64_t g = (work + block - 1) / block;
  if (g == 0) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

// ---- device helpers --------------------------------------------------------

// Loads that bypass L1 so that values written by other SMs during the same
// kernel are seen (L2 is the point of coherence).
__device__ __forceinline__ uint32_t ld_cg(const uint32_t *p) { return __ldcg(p); }
__device__ __forceinline__ uint64_t ld_cg(const uint64_t *p) {
  return __ldcg(reinterpret_cast<const unsigned long long *>(p));
}
__device__ __forceinline__ void st_cg(uint32_t *p, uint32_t v) { __stcg(p, v); }
__device__ __forceinline__ void st_cg(uint64_t *p, uint64_t v) {
  __stcg(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}

// ---- union-find in shared memory ----------------------------------------------
// Used by the tiled pass (uf.cu), the batched solve (batch.cu) and the server's
// small graphs (serve.cu).  A non-root entry always points at a smaller index,
// so the forest stays acyclic and each root is the smallest index of its tree;
// a find points every entry it passes at its grandparent.  Entries are 16 or
// 32 bits wide.
__device__ __forceinline__ uint32_t smem_cas(uint16_t *a, uint32_t c, uint32_t v) {
  return atomicCAS(reinterpret_cast<unsigned short *>(a), (unsigned short)c, (unsigned short)v);
}
__device__ __forceinline__ uint32_t smem_cas(uint32_t *a, uint32_t c, uint32_t v) {
  return atomicCAS(reinterpret_cast<unsigned int *>(a), c, v);
}
template <class PT>
__device__ __forceinline__ uint32_t smem_find(volatile PT *p, uint32_t v) {
  uint32_t cur = p[v];
  if (cur == v) return v;
  uint32_t prev = v, next;
  while (cur > (next = p[cur])) {
    p[prev] = (PT)next;
    prev = cur;
    cur = next;
  }
  return cur;
}
// Union of a and b: the larger root is CAS'ed under the smaller one.  With
// POINT_ENDS, both endpoints then point straight at the common root they saw
// (an ancestor of both, never a root that could still be CAS'ed: an endpoint
// other than that root has a parent already), so the next edges of a and b
// start next to the root.
template <bool POINT_ENDS, class PT>
__device__ __forceinline__ void smem_union(volatile PT *p, uint32_t a, uint32_t b) {
  uint32_t ra = smem_find(p, a), rb = smem_find(p, b);
  while (ra != rb) {
    if (ra < rb) {
      const uint32_t t = ra;
      ra = rb;
      rb = t;
    }
    const uint32_t old = smem_cas(const_cast<PT *>(p + ra), ra, rb);
    if (old == ra) {
      ra = rb;
      break;
    }
    ra = smem_find(p, old);
    rb = smem_find(p, rb);
  }
  if (POINT_ENDS) {
    if (a != ra) p[a] = (PT)ra;
    if (b != ra) p[b] = (PT)ra;
  }
}

template <class T>
__device__ __forceinline__ uint32_t load_id(const T *col, uint64_t e) {
  return (uint32_t)__ldg(col + e);
}

// Vertex -> virtual rank of the contiguous split n/P + (r < n%P)
// (graph_io.h:308-313).
struct PartMap {
  uint32_t q, rm, big;  // q = n/P, rm = n%P, big = rm*(q+1)
  __host__ __device__ PartMap() : q(0), rm(0), big(0) {}
  __host__ __device__ PartMap(uint64_t n, uint32_t P) {
    q = (uint32_t)(n / P);
    rm = (uint32_t)(n % P);
    big = rm * (q + 1);
  }
  __host__ __device__ __forceinline__ uint32_t part(uint32_t v) const {
    return v < big ? v / (q + 1) : rm + (q ? (v - big) / q : 0);
  }
  // [lo, hi) of v's rank: one division per row, so that a kernel tests an
  // edge's other end with two compares instead of a division per edge
  __host__ __device__ __forceinline__ void bounds(uint32_t v, uint32_t &lo, uint32_t &hi) const {
    const uint32_t r = part(v);
    lo = r < rm ? r * (q + 1) : big + (r - rm) * q;
    hi = lo + (r < rm ? q + 1 : q);
  }
};

// SplitMix64 finaliser: the counter-based hash behind every random variate.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
  return mix64(mix64(mix64(seed) ^ a) ^ (b * 0xd6e8feb86659fd93ull));
}

// a[l] = min(a[l], x) for the lanes with act set, called by all 32 lanes of
// the warp: lanes with the same l are merged first (one atomic per distinct l),
// and the atomic is skipped when a[l] already holds x or less.  Entries only
// decrease while the kernel runs, so a stale read is never below the true
// entry and a skip it allows is right; the read goes through L1 so that a
// label shared by many rows is not one L2 line every warp reads.
__device__ __forceinline__ void warp_min_to(uint32_t *a, bool act, uint32_t l, uint32_t x) {
  const unsigned am = __ballot_sync(0xffffffffu, act);
  if (!act) return;
  const unsigned peers = __match_any_sync(am, l);
  const uint32_t mn = __reduce_min_sync(peers, x);
  if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1) && mn < a[l]) atomicMin(a + l, mn);
}

// Warp-aggregated "any lane set" flag: one atomicOr per warp.
__device__ __forceinline__ void warp_flag(int pred, int *flag) {
  unsigned b = __ballot_sync(__activemask(), pred);
  if (b && (threadIdx.x & 31) == (unsigned)(__ffs(b) - 1)) atomicOr(flag, 1);
}

// Rows longer than a limit, as (row, piece) work items of kRowPiece entries:
// the sweeps hand each item to one warp, so a hub row of a hundred thousand
// entries is spread over many warps instead of holding one.
constexpr uint64_t kRowPiece = 2048;
inline uint64_t row_pieces_cap(uint64_t m, uint64_t limit) {
  return m / (limit + 1) + m / kRowPiece + 2;
}
struct RowPieces {
  uint2 *items;  // (row, piece index)
  uint64_t cap;
  unsigned int *count;
};
namespace {
// One reservation per warp (the warp's piece counts summed by a shuffle
// scan): a global atomic per long row serialised on the one counter, 1.2 ms
// for the 1.5 M rows above 64 entries of the 2^26-vertex hyperbolic graph.
// Launched with a multiple of 32 threads per block.
__global__ void k_row_pieces(uint64_t n, const uint64_t *__restrict__ rp, uint64_t limit,
                             RowPieces rpc) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); v0 < n; v0 += stride) {
    const uint64_t v = v0 + lane;  // v0 is the same for the whole warp
    uint32_t np = 0;
    if (v < n) {
      const uint64_t d = rp[v + 1] - rp[v];
      if (d > limit) np = (uint32_t)((d + kRowPiece - 1) / kRowPiece);
    }
    uint32_t inc = np;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if ((int)lane >= o) inc += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    if (total == 0) continue;  // warp-uniform
    unsigned int base = 0;
    if (lane == 31) base = atomicAdd(rpc.count, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    const uint64_t slot = (uint64_t)base + (inc - np);
    for (uint32_t q = 0; q < np && slot + q < rpc.cap; ++q)
      rpc.items[slot + q] = make_uint2((uint32_t)v, q);
  }
}
}  // namespace
// ---- row minimum with loads in flight ------------------------------------------
// The sweeps (label and shortcut rounds, decomposition relaxation, local
// contraction) take, for a row's entries [b, e), the minimum of a value
// gathered at each neighbour.  One thread walks its row four entries at a
// time: one 16-byte load of four ids (from the row's first 16-byte boundary
// on), then four independent gathers, so each thread keeps four dependent
// load chains in flight instead of one.  (A
// flattened 32-rows-per-warp stream was measured slower on the hyperbolic
// graph: its row search and segmented minimum cost about 20 shuffles per 32
// entries and left the kernel bound on the load/store pipe, while a thread's
// own row of about 16 ids sits in two sectors that L1 keeps.)
template <class V, class Gather>
__device__ __forceinline__ V row_min_ilp(const uint32_t *__restrict__ col, uint64_t b, uint64_t e,
                                         V best, Gather gather) {
  uint64_t j = b;
  // ids one at a time up to a 16-byte boundary, then four per load
  for (; j < e && (reinterpret_cast<uintptr_t>(col + j) & 15u); ++j) {
    const V x = gather(__ldg(col + j));
    best = x < best ? x : best;
  }
  for (; j + 4 <= e; j += 4) {
    const uint4 u = __ldg(reinterpret_cast<const uint4 *>(col + j));
    const V x0 = gather(u.x), x1 = gather(u.y), x2 = gather(u.z), x3 = gather(u.w);
    const V a = x0 < x1 ? x0 : x1, c = x2 < x3 ? x2 : x3, m = a < c ? a : c;
    best = m < best ? m : best;
  }
  for (; j < e; ++j) {
    const V x = gather(__ldg(col + j));
    best = x < best ? x : best;
  }
  return best;
}
// The same over a warp's piece [b, e) of a long row, lane-strided; the
// caller reduces over the warp.
template <class V, class Gather>
__device__ __forceinline__ V piece_min_ilp(const uint32_t *__restrict__ col, uint64_t b, uint64_t e,
                                           unsigned lane, V best, Gather gather) {
  uint64_t j = b + lane;
  for (; j + 96 < e; j += 128) {
    const uint32_t u0 = __ldg(col + j), u1 = __ldg(col + j + 32), u2 = __ldg(col + j + 64),
                   u3 = __ldg(col + j + 96);
    const V x0 = gather(u0), x1 = gather(u1), x2 = gather(u2), x3 = gather(u3);
    const V a = x0 < x1 ? x0 : x1, c = x2 < x3 ? x2 : x3, m = a < c ? a : c;
    best = m < best ? m : best;
  }
  for (; j < e; j += 32) {
    const V x = gather(__ldg(col + j));
    best = x < best ? x : best;
  }
  return best;
}

// Entries [b, e) of work item h.
__device__ __forceinline__ void row_piece(const RowPieces &rpc, const uint64_t *__restrict__ rp,
                                          uint64_t h, uint32_t &v, uint64_t &b, uint64_t &e) {
  const uint2 it = rpc.items[h];
  v = it.x;
  const uint64_t re = __ldg(rp + v + 1);
  b = __ldg(rp + v) + (uint64_t)it.y * kRowPiece;
  e = min(re, b + kRowPiece);
}

}  // namespace ccg

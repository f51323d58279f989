// ldd.cu - exponential-shift low-diameter decomposition and the local
// contraction sweeps.
//
// Reference: ExponentialContraction::RunContractionLP
// (exponential_contraction.h:439-628).  Every vertex draws a deviate
// dev = (u64)Exp(beta) (:469-472) and then repeatedly adopts
// (dev_w + 1, label_w) from a neighbour w when it is lexicographically
// smaller than its own (dev, label) (:527-549), until no vertex changes.  The
// fixpoint is  key(v) = min_u (dev_u + dist(u, v), label_u),  which does not
// depend on the update order, so the decomposition (each vertex's centre) is
// fully determined by the deviates.
//
// GB300 layout: one 64-bit key per vertex, (dev << 32) | index.  Vertex
// indices of every level graph are numbered in increasing original-id order,
// so comparing indices compares the reference's labels, and adding 2^32 is
// the "+1" on the deviate.  A relaxation is then a u64 min; the centre is the
// low word of the key.
//
// Deviates: the reference draws from std::exponential_distribution seeded per
// vertex with a std::default_random_engine (:469-472).  Here a counter-based
// hash of (seed, original id, level) gives a uniform 64-bit word u, and
// dev = #{k >= 1 : u < T[k]} with T[k] = floor(2^64 exp(-beta k)): inverse
// transform sampling of floor(Exp(beta)), which is geometric with
// P(dev >= k) = exp(-beta k).  T is built on the host with a fixed sequence
// of IEEE double operations (det_exp below), so the table, and with it every
// deviate, is the same on every host.
#include <cmath>
#include <vector>

#include "kernels.h"

namespace ccg {
// Sweeps bound to eight CTAs of 256 threads per SM (32 registers): the
// id-checking first sweep had taken 38 registers, six CTAs per SM, and this
// latency-bound gather runs faster with the two extra CTAs (local
// contraction's sweeps on the 2^26 hyperbolic graph: 6.2 -> 5.9 ms).
constexpr int kSweepCtasPerSM = 8;

// exp(x) for x <= 0 from range reduction by ln 2 and a Taylor series, with a
// fixed evaluation order (no library call, no contraction into FMA), so that
// the result is identical on every IEEE-754 host.
double det_exp(double x) {
  const double ln2 = 0.6931471805599453094172321;
  double kf = std::floor(x / ln2 + 0.5);
  volatile double r = x - kf * ln2;  // volatile: keep the two roundings
  double rr = r;
  double term = 1.0, sum = 1.0;
  for (int i = 1; i < 30; ++i) {
    term = term * rr;
    term = term / (double)i;
    sum = sum + term;
  }
  return std::ldexp(sum, (int)kf);
}

int geo_table_build(double beta, std::vector<uint64_t> &t) {
  t.clear();
  if (!(beta > 0.0)) return 0;
  const int kmax = 4096;
  for (int k = 1; k <= kmax; ++k) {
    double p = det_exp(-beta * (double)k);
    double x = std::ldexp(p, 64);
    if (x < 1.0) break;
    uint64_t v = x >= 18446744073709551615.0 ? ~0ull : (uint64_t)x;
    t.push_back(v);
  }
  return (int)t.size();
}

namespace {

__device__ __forceinline__ uint32_t geo_dev(uint64_t u, const uint64_t *__restrict__ T, int len) {
  // T is non-increasing: {k : u < T[k-1]} is a prefix 1..j; find j.
  int lo = 0, hi = len;  // answer in [lo, hi]
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (u < __ldg(T + mid - 1)) lo = mid;
    else hi = mid - 1;
  }
  return (uint32_t)lo;
}

__global__ void k_ldd_init(uint64_t n, const uint32_t *__restrict__ vid, uint64_t seed,
                           uint32_t level, const uint64_t *__restrict__ T, int len,
                           uint64_t *__restrict__ key, unsigned int *__restrict__ maxdev) {
  uint32_t mx = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t u = hash3(seed, vid[i], level);
    uint32_t d = geo_dev(u, T, len);
    key[i] = ((uint64_t)d << 32) | (uint32_t)i;
    mx = d > mx ? d : mx;
  }
  for (int o = 16; o; o >>= 1) {
    uint32_t y = __shfl_xor_sync(__activemask(), mx, o);
    mx = y > mx ? y : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(maxdev, mx);
}

constexpr uint64_t kOne = 1ull << 32;
constexpr uint64_t kRowLimit = 64;  // rows above this are relaxed a warp per piece

// One Gauss-Seidel style sweep: key[v] <- min(key[v], min_w key[w] + 2^32).
// Stale neighbour reads are upper bounds of the fixpoint, so in-place updates
// converge to the same keys as the reference's sweeps.
__global__ void k_ldd_round(uint64_t n, const uint64_t *__restrict__ rp,
                            const uint32_t *__restrict__ col, uint64_t *key, int *flag) {
  int changed = 0;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    if (e - b > kRowLimit) continue;
    const uint64_t k = ld_cg(key + v);
    const uint64_t best =
        row_min_ilp<uint64_t>(col, b, e, k, [&](uint32_t u) { return ld_cg(key + u) + kOne; });
    if (best < k) {
      st_cg(key + v, best);
      changed = 1;
    }
  }
  warp_flag(changed, flag);
}

// Rows above kRowLimit entries, one warp per piece of the row.
__global__ void k_ldd_round_pieces(const uint64_t *__restrict__ rp, const uint32_t *__restrict__ col,
                                   RowPieces rpc, uint64_t *key, int *flag) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t ni = min((uint64_t)*rpc.count, rpc.cap);
  int changed = 0;
  for (uint64_t h = warp; h < ni; h += nwarps) {
    uint32_t v;
    uint64_t b, e;
    row_piece(rpc, rp, h, v, b, e);
    uint64_t best = piece_min_ilp<uint64_t>(col, b, e, lane, ~0ull,
                                            [&](uint32_t u) { return ld_cg(key + u) + kOne; });
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      uint64_t y = __shfl_xor_sync(0xffffffffu, best, o);
      best = y < best ? y : best;
    }
    if (lane == 0) {
      uint64_t k = ld_cg(key + v);
      if (best < k) {
        atomicMin(reinterpret_cast<unsigned long long *>(key + v), (unsigned long long)best);
        changed = 1;
      }
    }
  }
  warp_flag(changed, flag);
}

// Start-time gated round t (RunContractionBFS, exponential_contraction.h:
// 630-859): vertices whose key has deviate part t are final and push
// key + 2^32 to their neighbours.  Ties are broken by label, as in the
// sweeps, so both variants reach the same keys.
__global__ void k_ldd_gated(uint64_t n, const uint64_t *__restrict__ rp,
                            const uint32_t *__restrict__ col, uint64_t *key, uint32_t t) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t k = ld_cg(key + v);
    if ((uint32_t)(k >> 32) != t) continue;
    uint64_t kp = k + kOne;
    uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    for (uint64_t j = b; j < e; ++j) {
      uint32_t w = __ldg(col + j);
      if (ld_cg(key + w) > kp)
        atomicMin(reinterpret_cast<unsigned long long *>(key + w), (unsigned long long)kp);
    }
  }
}

__global__ void k_low_word(uint64_t n, const uint64_t *__restrict__ key, uint32_t *__restrict__ cl) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    cl[i] = (uint32_t)key[i];
}

// ---- local contraction (local_contraction.h:157-300) -----------------------
// The sweeps take the minimum of the key (d, i) (deviate, then index) over a
// neighbourhood, and the cluster is the index of that minimum.  Only the
// order of the keys matters, so the sweeps run on each key's rank in that
// order, a 32-bit value (a 4-byte gather per entry instead of 8), and the
// index is read back through the inverse map.  The ranks are the stable ranks
// of the deviates (ties in index order).
__global__ void k_local_init(uint64_t n, const uint32_t *__restrict__ vid, uint64_t seed,
                             uint32_t level, uint8_t *__restrict__ dig) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    // uniform integer in [0, 99] (reference: uniform_int_distribution(0, 99))
    dig[i] = (uint8_t)(((hash3(seed, vid[i], level) >> 32) * 100ull) >> 32);
  }
}
__global__ void k_local_clusters(uint64_t n, const uint32_t *__restrict__ best,
                                 const uint32_t *__restrict__ inv, uint32_t *__restrict__ cl) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    cl[v] = inv[best[v]];
}

// Jacobi sweep: out[v] = min over N[v] (closed neighbourhood) of in[].  Rows
// above kRowLimit entries only store in[v] here; k_min_sweep_pieces folds
// their neighbours in afterwards, one warp per piece of the row.
// CHECK (the first sweep over a caller's ids that no pass has checked): an id
// >= n is skipped and recorded in *err, which the host reads before any
// kernel trusts the ids.
template <bool CHECK>
__global__ void __launch_bounds__(kBlock, kSweepCtasPerSM) k_min_sweep(uint64_t n, const uint64_t *__restrict__ rp,
                            const uint32_t *__restrict__ col, const uint32_t *__restrict__ in,
                            uint32_t *__restrict__ out, int *err) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    uint32_t best = in[v];
    bool bad = false;
    if (e - b <= kRowLimit)
      best = row_min_ilp<uint32_t>(col, b, e, best, [&](uint32_t u) {
        if (CHECK && u >= n) {
          bad = true;
          return kNone;
        }
        return __ldg(in + u);
      });
    if (CHECK && bad) set_err(err, kErrBadId);
    out[v] = best;
  }
}

template <bool CHECK>
__global__ void k_min_sweep_pieces(uint64_t n, const uint64_t *__restrict__ rp,
                                   const uint32_t *__restrict__ col, RowPieces rpc,
                                   const uint32_t *__restrict__ in, uint32_t *out, int *err) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t ni = min((uint64_t)*rpc.count, rpc.cap);
  for (uint64_t h = warp; h < ni; h += nwarps) {
    uint32_t v;
    uint64_t b, e;
    row_piece(rpc, rp, h, v, b, e);
    bool bad = false;
    uint32_t best = piece_min_ilp<uint32_t>(col, b, e, lane, kNone, [&](uint32_t u) {
      if (CHECK && u >= n) {
        bad = true;
        return kNone;
      }
      return __ldg(in + u);
    });
    if (CHECK && bad) set_err(err, kErrBadId);
    best = __reduce_min_sync(0xffffffffu, best);
    if (lane == 0) atomicMin(out + v, best);
  }
}

}  // namespace

void geo_table_upload(double beta, uint64_t *d_table, int *len_out, cudaStream_t s) {
  std::vector<uint64_t> t;
  int len = geo_table_build(beta, t);
  if (len) CCG_CUDA(cudaMemcpyAsync(d_table, t.data(), 8 * len, cudaMemcpyHostToDevice, s));
  CCG_CUDA(cudaStreamSynchronize(s));  // t is a host temporary
  *len_out = len;
}

int ldd_decompose(const Csr &g, const uint32_t *vid, uint64_t seed, uint32_t level,
                  const uint64_t *d_geo, int geo_len, bool gated, uint32_t *cluster,
                  uint64_t *key, int max_rounds, cudaStream_t s, cudaMemPool_t pool,
                  Counters &c, volatile int *host_flag, int *dev_flag) {
  if (g.n == 0) return 0;
  const uint32_t *col = static_cast<const uint32_t *>(g.col);
  unsigned grid = grid_for(g.n, kBlock, num_sms() * 32);
  DevBuf mx(4, s, pool);
  CCG_CUDA(cudaMemsetAsync(mx.p, 0, 4, s));
  k_ldd_init<<<grid, kBlock, 0, s>>>(g.n, vid, seed, level, d_geo, geo_len, key,
                                     mx.as<unsigned int>());
  CCG_LAUNCH_CHECK();
  c.add(1, 4 * g.n + 8 * g.n);
  int rounds = 0;
  const uint64_t round_bytes = 8 * (g.n + 1) + g.m * 4 + g.m * 8 + 2 * g.n * 8;
  if (gated) {
    uint32_t maxdev = 0;
    CCG_CUDA(cudaMemcpyAsync(&maxdev, mx.p, 4, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    cudaEvent_t t0 = c.tic(s);
    for (uint32_t t = 0; t <= maxdev; ++t) {
      k_ldd_gated<<<grid, kBlock, 0, s>>>(g.n, g.rp, col, key, t);
      CCG_LAUNCH_CHECK();
      ++rounds;
    }
    c.toc(s, "ldd_gated_all_rounds", t0,
          8 * (g.n + 1) + g.m * 4 + g.m * 8 + (uint64_t)rounds * g.n * 8);
    // every vertex is final once; every edge pushed once
    c.add(rounds, 8 * (g.n + 1) + g.m * 4 + g.m * 8 + (uint64_t)rounds * g.n * 8);
  } else {
    const uint64_t cap = row_pieces_cap(g.m, kRowLimit);
    DevBuf items(8 * cap, s, pool), cnt(4, s, pool);
    CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 4, s));
    const RowPieces rpc{items.as<uint2>(), cap, cnt.as<unsigned int>()};
    k_row_pieces<<<grid, kBlock, 0, s>>>(g.n, g.rp, kRowLimit, rpc);
    CCG_LAUNCH_CHECK();
    for (;;) {
      if (rounds >= max_rounds) return -1;
      *host_flag = 0;
      CCG_CUDA(cudaMemsetAsync(dev_flag, 0, sizeof(int), s));
      cudaEvent_t t0 = c.tic(s);
      k_ldd_round<<<grid, kBlock, 0, s>>>(g.n, g.rp, col, key, dev_flag);
      CCG_LAUNCH_CHECK();
      k_ldd_round_pieces<<<num_sms() * 8, kBlock, 0, s>>>(g.rp, col, rpc, key, dev_flag);
      CCG_LAUNCH_CHECK();
      c.toc(s, "ldd_round", t0, round_bytes);
      CCG_CUDA(cudaMemcpyAsync((void *)host_flag, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      CCG_CUDA(cudaStreamSynchronize(s));
      ++rounds;
      c.add(2, round_bytes);
      if (*host_flag == 0) break;
    }
  }
  k_low_word<<<grid, kBlock, 0, s>>>(g.n, key, cluster);
  CCG_LAUNCH_CHECK();
  c.add(1, 12 * g.n);
  return rounds;
}

void local_sweeps(const Csr &g, const uint32_t *vid, uint64_t seed, uint32_t level,
                  uint32_t *cluster, cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  if (g.n == 0) return;
  const uint32_t *col = static_cast<const uint32_t *>(g.col);
  unsigned grid = grid_for(g.n, kBlock, num_sms() * 32);
  const uint64_t cap = row_pieces_cap(g.m, kRowLimit);
  DevBuf items(8 * cap, s, pool), cnt(4, s, pool), rank(4 * g.n, s, pool), best(4 * g.n, s, pool),
      inv(4 * g.n, s, pool), digits(g.n, s, pool);
  CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 4, s));
  const RowPieces rpc{items.as<uint2>(), cap, cnt.as<unsigned int>()};
  cudaEvent_t tr = c.tic(s);
  uint8_t *dig = digits.as<uint8_t>();
  k_local_init<<<grid, kBlock, 0, s>>>(g.n, vid, seed, level, dig);
  CCG_LAUNCH_CHECK();
  stable_digit_ranks(dig, g.n, rank.as<uint32_t>(), inv.as<uint32_t>(), s, pool, c);
  c.toc(s, "local_rank", tr, 4 * g.n + g.n + 2 * g.n + 8 * g.n);
  c.add(1, 4 * g.n + g.n);
  cudaEvent_t t0 = c.tic(s);
  k_row_pieces<<<grid, kBlock, 0, s>>>(g.n, g.rp, kRowLimit, rpc);
  CCG_LAUNCH_CHECK();
  for (int r = 0; r < 2; ++r) {  // N(v), then N(N(v))
    const uint32_t *in = r ? best.as<uint32_t>() : rank.as<uint32_t>();
    uint32_t *out = r ? rank.as<uint32_t>() : best.as<uint32_t>();
    if (r == 0 && g.err) {  // the caller's ids, not checked yet
      k_min_sweep<true><<<grid, kBlock, 0, s>>>(g.n, g.rp, col, in, out, g.err);
      CCG_LAUNCH_CHECK();
      k_min_sweep_pieces<true><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.rp, col, rpc, in, out,
                                                                g.err);
    } else {
      k_min_sweep<false><<<grid, kBlock, 0, s>>>(g.n, g.rp, col, in, out, nullptr);
      CCG_LAUNCH_CHECK();
      k_min_sweep_pieces<false><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.rp, col, rpc, in, out,
                                                                 nullptr);
    }
    CCG_LAUNCH_CHECK();
  }
  const uint64_t sweep = 8 * (g.n + 1) + g.m * 4 + g.m * 4 + 2 * g.n * 4;
  c.toc(s, "local_sweeps", t0, 2 * sweep);
  k_local_clusters<<<grid, kBlock, 0, s>>>(g.n, rank.as<uint32_t>(), inv.as<uint32_t>(), cluster);
  CCG_LAUNCH_CHECK();
  c.add(6, 12 * g.n + 2 * sweep);
}

}  // namespace ccg

// gen_dev.cu - the seeded G(n, m) and 2D bond-percolation generators on the
// device: the same graphs as the host generators of csrc/gen.cpp (the same
// SplitMix64 hash of (seed, index, stream), the same rows in the same order),
// built where the solver will read them, without a host copy.  Stand-ins for
// the KaGen generators of the reference drivers (lib/io/io_utils.h:59-83).
#include <algorithm>
#include <cmath>

#include "../../include/cc_gpu.h"
#include "ctx.h"

namespace ccg {
namespace {

// uniform integer in [0, n) from the high word (n < 2^32), as on the host
__device__ __forceinline__ uint64_t below(uint64_t h, uint64_t n) { return ((h >> 32) * n) >> 32; }

struct GridEdges {
  uint64_t X, Y, seed, thr;
  bool all, none;
  __device__ __forceinline__ bool right(uint64_t v) const {  // edge v -- v+1 (same row)
    return (v % X) + 1 < X && (all || (!none && hash3(seed, v, 0) < thr));
  }
  __device__ __forceinline__ bool down(uint64_t v) const {  // edge v -- v+X
    return v / X + 1 < Y && (all || (!none && hash3(seed, v, 1) < thr));
  }
};

__global__ void k_grid_degrees(GridEdges ge, uint8_t *__restrict__ deg) {
  const uint64_t n = ge.X * ge.Y;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t x = v % ge.X;
    deg[v] = (uint8_t)((v >= ge.X && ge.down(v - ge.X)) + (x > 0 && ge.right(v - 1)) + ge.right(v) +
                       ge.down(v));
  }
}

// rows sorted: up, left, right, down
template <class T>
__global__ void k_grid_fill(GridEdges ge, const uint64_t *__restrict__ rp, T *__restrict__ col) {
  const uint64_t n = ge.X * ge.Y;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t x = v % ge.X;
    uint64_t e = rp[v];
    if (v >= ge.X && ge.down(v - ge.X)) col[e++] = (T)(v - ge.X);
    if (x > 0 && ge.right(v - 1)) col[e++] = (T)(v - 1);
    if (ge.right(v)) col[e++] = (T)(v + 1);
    if (ge.down(v)) col[e++] = (T)(v + ge.X);
  }
}

// both directions of every drawn pair as (src << b) | dst; self-loops become
// ~0, whose low 2b bits sort after every pair key (the largest pair key,
// ((n-1) << b) | (n-2), is below 2^(2b) - 1)
__global__ void k_gnm_keys(uint64_t n, uint64_t m, uint64_t seed, int b, uint64_t *__restrict__ keys) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t u = below(hash3(seed, i, 1), n), w = below(hash3(seed, i, 2), n);
    keys[2 * i] = u == w ? ~0ull : (u << b) | w;
    keys[2 * i + 1] = u == w ? ~0ull : (w << b) | u;
  }
}

// rp[v] = first key with source >= v (v in [0, n]); col = the keys' targets
template <class T>
__global__ void k_keys_to_csr(const uint64_t *__restrict__ keys, uint64_t nk, uint64_t n, int b,
                              uint64_t *__restrict__ rp, T *__restrict__ col) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (uint64_t v = t; v <= n; v += stride) {
    uint64_t lo = 0, hi = nk;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if ((keys[mid] >> b) < v) lo = mid + 1;
      else hi = mid;
    }
    rp[v] = lo;
  }
  const uint64_t mask = (1ull << b) - 1;
  for (uint64_t e = t; e < nk; e += stride) col[e] = (T)(keys[e] & mask);
}

int bits_for_n(uint64_t x) {
  int b = 1;
  while (b < 64 && (1ull << b) < x) ++b;
  return b;
}

}  // namespace
}  // namespace ccg

using ccg::DevBuf;
using ccg::Error;

extern "C" {

int cc_gen_grid_device(cc_ctx *ctx, uint64_t X, uint64_t Y, double p, uint64_t seed, uint32_t id_bytes,
                       uint64_t *row_ptr, void *col, uint64_t cap, uint64_t *m_dir) {
  return ccg::guard([&] {
    if ((id_bytes != 4 && id_bytes != 8) || X == 0 || Y == 0 || !row_ptr || !m_dir || (cap && !col))
      throw Error(CC_ERR_INVALID, "bad grid generator arguments");
    const uint64_t n = X * Y;
    if (n / X != Y || n >= (1ull << 30))  // offsets are rebuilt with a 32-bit scan (<= 4n entries)
      throw Error(CC_ERR_UNSUPPORTED, "grid of 2^30 vertices or more");
    cc_ctx *C = ctx ? ctx : ccg::default_context();
    CCG_CUDA(cudaSetDevice(C->device));
    cudaStream_t s = C->stream;
    ccg::Counters c;
    const bool all = p >= 1.0, none = p <= 0.0;
    const ccg::GridEdges ge{X, Y, seed, (all || none) ? 0ull : (uint64_t)std::ldexp(p, 64), all, none};
    DevBuf deg(n, s, C->pool);
    const unsigned grid = ccg::grid_for(n, ccg::kBlock, ccg::num_sms() * 16);
    ccg::k_grid_degrees<<<grid, ccg::kBlock, 0, s>>>(ge, deg.as<uint8_t>());
    CCG_LAUNCH_CHECK();
    ccg::offsets_from_degrees(deg.as<uint8_t>(), n, 0, row_ptr, s, C->pool, c);
    uint64_t m = 0;
    CCG_CUDA(cudaMemcpyAsync(&m, row_ptr + n, 8, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    *m_dir = m;
    if (m > cap) throw Error(CC_ERR_INVALID, "col capacity below the generated entries");
    if (id_bytes == 8)
      ccg::k_grid_fill<uint64_t><<<grid, ccg::kBlock, 0, s>>>(ge, row_ptr, static_cast<uint64_t *>(col));
    else
      ccg::k_grid_fill<uint32_t><<<grid, ccg::kBlock, 0, s>>>(ge, row_ptr, static_cast<uint32_t *>(col));
    CCG_LAUNCH_CHECK();
    CCG_CUDA(cudaStreamSynchronize(s));
  });
}

int cc_gen_gnm_device(cc_ctx *ctx, uint64_t n, uint64_t m, uint64_t seed, uint32_t id_bytes,
                      uint64_t *row_ptr, void *col, uint64_t cap, uint64_t *m_dir) {
  return ccg::guard([&] {
    if ((id_bytes != 4 && id_bytes != 8) || n == 0 || n >= (1ull << 32) || !row_ptr || !m_dir ||
        (cap && !col))
      throw Error(CC_ERR_INVALID, "bad G(n, m) generator arguments");
    if (2 * m >= (1ull << 32)) throw Error(CC_ERR_UNSUPPORTED, "2m >= 2^32 directed entries");
    cc_ctx *C = ctx ? ctx : ccg::default_context();
    CCG_CUDA(cudaSetDevice(C->device));
    cudaStream_t s = C->stream;
    ccg::Counters c;
    const int b = ccg::bits_for_n(n);
    const uint64_t nk = 2 * m;
    DevBuf keys(8 * (nk ? nk : 1), s, C->pool), tmp(8 * (nk ? nk : 1), s, C->pool),
        uniq(8 * (nk ? nk : 1), s, C->pool), cnt(4, s, C->pool);
    uint64_t u = 0;
    const uint64_t *sorted = keys.as<uint64_t>();
    if (nk) {
      ccg::k_gnm_keys<<<ccg::grid_for(m, ccg::kBlock, ccg::num_sms() * 16), ccg::kBlock, 0, s>>>(
          n, m, seed, b, keys.as<uint64_t>());
      CCG_LAUNCH_CHECK();
      sorted = ccg::radix_sort_u64(keys.as<uint64_t>(), tmp.as<uint64_t>(), nk, 2 * b, s, C->pool, c);
      ccg::unique_sorted_keys(sorted, nk, uniq.as<uint64_t>(), cnt.as<uint32_t>(), s, C->pool, c);
      uint32_t nu = 0;
      uint64_t last = 0;
      CCG_CUDA(cudaMemcpyAsync(&nu, cnt.p, 4, cudaMemcpyDeviceToHost, s));
      CCG_CUDA(cudaStreamSynchronize(s));
      if (nu) {
        CCG_CUDA(cudaMemcpyAsync(&last, uniq.as<uint64_t>() + nu - 1, 8, cudaMemcpyDeviceToHost, s));
        CCG_CUDA(cudaStreamSynchronize(s));
      }
      u = nu - (nu && last == ~0ull ? 1 : 0);  // the self-loop marker, sorted last
    }
    *m_dir = u;
    if (u > cap) throw Error(CC_ERR_INVALID, "col capacity below the generated entries");
    const unsigned grid = ccg::grid_for(std::max<uint64_t>(n + 1, u), ccg::kBlock, ccg::num_sms() * 16);
    if (id_bytes == 8)
      ccg::k_keys_to_csr<uint64_t><<<grid, ccg::kBlock, 0, s>>>(uniq.as<uint64_t>(), u, n, b, row_ptr,
                                                                static_cast<uint64_t *>(col));
    else
      ccg::k_keys_to_csr<uint32_t><<<grid, ccg::kBlock, 0, s>>>(uniq.as<uint64_t>(), u, n, b, row_ptr,
                                                                static_cast<uint32_t *>(col));
    CCG_LAUNCH_CHECK();
    CCG_CUDA(cudaStreamSynchronize(s));
  });
}

}  // extern "C"

// scan.cuh - the three-phase exclusive scan over a value functor, shared by
// the files that compact or scan on the device (sortcsr.cu, load_dev.cu).
// Phase 1: per-tile sums.  Phase 2: scan of the tile sums (recursive).
// Phase 3: per-tile scan plus the tile offset, handed to a writer functor.
// Sums are 32-bit: one call covers fewer than 2^32 in total.
#pragma once

#include "kernels.h"

namespace ccg {
namespace {

constexpr int kScanItems = 8;
constexpr int kScanTile = kBlock * kScanItems;  // 2048 elements per block

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

// Exclusive block scan of one value per thread (blockDim == 256).
template <class T>
__device__ __forceinline__ T block_excl_scan(T x, T *sw, T &total) {
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  T inc = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= (unsigned)d) inc += y;
  }
  if (lane == 31) sw[w] = inc;
  __syncthreads();
  if (w == 0) {
    T s = lane < 8 ? sw[lane] : T(0);
#pragma unroll
    for (int d = 1; d < 8; d <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= (unsigned)d) s += y;
    }
    if (lane < 8) sw[lane] = s;
  }
  __syncthreads();
  T woff = w ? sw[w - 1] : T(0);
  total = sw[7];
  __syncthreads();
  return woff + inc - x;
}

template <class Get>
__global__ void k_tile_sum(uint64_t n, Get get, uint32_t *__restrict__ tile_sums) {
  __shared__ uint32_t sw[8];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += get(base + i);
  uint32_t total;
  block_excl_scan<uint32_t>(s, sw, total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

template <class Get, class Put>
__global__ void k_tile_scan(uint64_t n, Get get, Put put, const uint32_t *__restrict__ tile_offs) {
  __shared__ uint32_t sw[8];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t vals[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    vals[i] = (base + i < n) ? get(base + i) : 0u;
    s += vals[i];
  }
  uint32_t total;
  uint32_t run = block_excl_scan<uint32_t>(s, sw, total) + tile_offs[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) put(base + i, run, vals[i]);
    run += vals[i];
  }
}

struct GetArr {
  const uint32_t *a;
  __device__ uint32_t operator()(uint64_t i) const { return a[i]; }
};
struct PutArr {
  uint32_t *o;
  __device__ void operator()(uint64_t i, uint32_t excl, uint32_t) const { o[i] = excl; }
};

// In-place capable exclusive scan of uint32 -> uint32; *d_total (if given)
// receives the sum.
template <class Get, class Put>
void scan_generic(uint64_t n, Get get, Put put, uint32_t *d_total, cudaStream_t s,
                  cudaMemPool_t pool, Counters &c);

__global__ void k_set_total(const uint32_t *tile_offs, const uint32_t *tile_sums, uint64_t nt,
                            uint32_t *d_total) {
  *d_total = tile_offs[nt - 1] + tile_sums[nt - 1];
}

template <class Get, class Put>
void scan_generic(uint64_t n, Get get, Put put, uint32_t *d_total, cudaStream_t s,
                  cudaMemPool_t pool, Counters &c) {
  if (n == 0) {
    if (d_total) CCG_CUDA(cudaMemsetAsync(d_total, 0, 4, s));
    return;
  }
  uint64_t nt = (n + kScanTile - 1) / kScanTile;
  DevBuf sums(4 * nt, s, pool), offs(4 * nt, s, pool);
  k_tile_sum<<<(unsigned)nt, kBlock, 0, s>>>(n, get, sums.as<uint32_t>());
  CCG_LAUNCH_CHECK();
  if (nt == 1) {
    CCG_CUDA(cudaMemsetAsync(offs.p, 0, 4, s));
  } else {
    scan_generic(nt, GetArr{sums.as<uint32_t>()}, PutArr{offs.as<uint32_t>()}, nullptr, s, pool, c);
  }
  k_tile_scan<<<(unsigned)nt, kBlock, 0, s>>>(n, get, put, offs.as<uint32_t>());
  CCG_LAUNCH_CHECK();
  if (d_total) {
    k_set_total<<<1, 1, 0, s>>>(offs.as<uint32_t>(), sums.as<uint32_t>(), nt, d_total);
    CCG_LAUNCH_CHECK();
  }
  c.add(3, 0);
}

}  // namespace
}  // namespace ccg

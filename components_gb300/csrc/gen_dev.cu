// gen_dev.cu - the seeded G(n, m) and 2D bond-percolation generators on the
// device: the same graphs as the host generators of csrc/gen.cpp (the same
// SplitMix64 hash of (seed, index, stream), the same rows in the same order),
// built where the solver will read them, without a host copy.  Stand-ins for
// the KaGen generators of the reference drivers (lib/io/io_utils.h:59-83).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/cc_gpu.h"
#include "ctx.h"
#include "rhg.h"

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

// ---- random hyperbolic graph (rhg.h holds the model and the exact test) ----
// Points are kept as structure-of-arrays in the vertex (angular) order.
struct RhgPts {
  double *a, *b, *s, *x, *y;
  uint64_t *phi;
  uint32_t *band;
  __device__ __forceinline__ rhg::Point get(uint64_t v) const {
    rhg::Point p;
    p.a = a[v];
    p.b = b[v];
    p.s = s[v];
    p.x = x[v];
    p.y = y[v];
    p.phi = phi[v];
    p.band = (int)band[v];
    return p;
  }
};
// Per band: its vertices in increasing id (bl + band_start[b] ..), and its
// 2^L[b] + 1 cell starts (absolute positions in bl) at cell_off[b].
struct RhgBands {
  const uint32_t *bl;
  const uint64_t *band_start;  // nb + 1
  const uint64_t *cell;        // all bands' cell starts
  const uint64_t *cell_off;    // nb
  const int *L;                // nb
};

__global__ void k_rhg_keys(rhg::Params P, uint64_t *__restrict__ keys) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < P.n;
       i += (uint64_t)gridDim.x * blockDim.x)
    keys[i] = rhg::angle_key(P, i);
}

// points in vertex order, and the band keys (band << 32) | v for grouping
__global__ void k_rhg_points(rhg::Params P, const uint64_t *__restrict__ keys, RhgPts pt,
                             uint64_t *__restrict__ bkeys) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < P.n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const rhg::Point p = rhg::point(P, keys[v]);
    pt.a[v] = p.a;
    pt.b[v] = p.b;
    pt.s[v] = p.s;
    pt.x[v] = p.x;
    pt.y[v] = p.y;
    pt.phi[v] = p.phi;
    pt.band[v] = (uint32_t)p.band;
    bkeys[v] = ((uint64_t)p.band << 32) | v;
  }
}

// band_start[b] = first sorted band key of band >= b, b in [0, nb]
__global__ void k_rhg_band_starts(const uint64_t *__restrict__ bkeys, uint64_t n, int nb,
                                  uint64_t *__restrict__ band_start, uint32_t *__restrict__ bl) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (t <= (uint64_t)nb) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if ((bkeys[mid] >> 32) < t) lo = mid + 1;
      else hi = mid;
    }
    band_start[t] = lo;
  }
  for (uint64_t i = t; i < n; i += (uint64_t)gridDim.x * blockDim.x) bl[i] = (uint32_t)bkeys[i];
}

// Cell starts: entry j of band b = the first position of the band whose cell
// is >= j.  Inside a band the vertices are in increasing angle, so the cells
// are non-decreasing along the band: position k writes the entries of the
// cells from just after its predecessor's cell up to its own (and the last
// position of a band those after its own).  gk: the sorted (band << 32) | v
// keys; threads t < nb fill empty bands.
__global__ void k_rhg_cells(RhgBands B, RhgPts pt, const uint64_t *__restrict__ gk, uint64_t n,
                            int nb, uint64_t *__restrict__ cell) {
  const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (t0 < (uint64_t)nb && B.band_start[t0] == B.band_start[t0 + 1]) {
    const uint64_t cnt = (1ull << B.L[t0]) + 1;
    for (uint64_t j = 0; j < cnt; ++j) cell[B.cell_off[t0] + j] = B.band_start[t0];
  }
  for (uint64_t k = t0; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const int b = (int)(gk[k] >> 32);
    const int L = B.L[b];
    uint64_t *c = cell + B.cell_off[b];
    const uint64_t ck = rhg::cell_of(pt.phi[(uint32_t)gk[k]], L);
    const bool first = k == B.band_start[b], last = k + 1 == B.band_start[b + 1];
    const uint64_t from = first ? 0 : rhg::cell_of(pt.phi[(uint32_t)gk[k - 1]], L) + 1;
    for (uint64_t j = from; j <= ck; ++j) c[j] = k;
    if (last)
      for (uint64_t j = ck + 1; j <= (1ull << L); ++j) c[j] = k + 1;
  }
}

// Candidate positions of v in band b: one or two ranges [r[0], r[1]) and
// [r[2], r[3]) of bl; *win/*half describe the angular window (no window: the
// whole band).
__device__ __forceinline__ void rhg_band_ranges(const rhg::Params &P, const rhg::Point &pv,
                                                double inv_s, const RhgBands &B, int b,
                                                uint64_t r[4], bool *win, uint64_t *half) {
  const uint64_t bs = B.band_start[b], be = B.band_start[b + 1];
  r[0] = r[1] = r[2] = r[3] = bs;
  *win = false;
  *half = 0;
  if (bs == be) return;
  const int L = B.L[b];
  *win = L > 0 && rhg::window(P, pv, b, inv_s, half);
  if (!*win) {
    r[1] = be;
    return;
  }
  const uint64_t lo = pv.phi - *half, hi = pv.phi + *half;
  const uint64_t *c = B.cell + B.cell_off[b];
  const uint64_t c0 = rhg::cell_of(lo, L), c1 = rhg::cell_of(hi, L);
  if (lo > pv.phi || hi < pv.phi) {  // the window crosses angle 0
    r[0] = c[c0];
    r[1] = be;
    r[2] = bs;
    r[3] = c[c1 + 1];
  } else {
    r[0] = c[c0];
    r[1] = c[c1 + 1];
  }
}

// Candidate w of v: a neighbour?
__device__ __forceinline__ bool rhg_is_neighbour(const rhg::Params &P, const rhg::Point &pv, uint64_t v,
                                                 bool win, uint64_t half, const RhgPts &pt, uint32_t w) {
  if (w == v) return false;
  if (win && pt.phi[w] - (pv.phi - half) > 2 * half) return false;
  return rhg::adjacent(P, pv, pt.get(w));
}

// A vertex near the centre of the disk has candidates in the millions (the
// whole inner bands, wide windows in the outer ones); one thread would walk
// them alone for seconds.  Vertices with more than kRhgHeavy candidates go to
// a list and are searched by a whole block each (k_rhg_heavy).
constexpr uint64_t kRhgHeavy = 4096;

// Every neighbour of v (the candidate search of the host generator), one
// thread per vertex: with out == nullptr count them into deg[v], else write
// (v << idbits) | w keys from out[rp[v]].  Heavy vertices are skipped (the
// counting pass lists them in heavy / nheavy).
__global__ void k_rhg_neighbours(rhg::Params P, RhgPts pt, RhgBands B, uint32_t *__restrict__ deg,
                                 const uint64_t *__restrict__ rp, uint64_t *__restrict__ out,
                                 uint32_t *__restrict__ heavy, unsigned int *__restrict__ nheavy) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < P.n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const rhg::Point pv = pt.get(v);
    const double inv_s = pv.s > 0.0 ? 1.0 / pv.s : 0.0;
    uint64_t est = 0;
    for (int b = 0; b < P.nb && est <= kRhgHeavy; ++b) {
      uint64_t r[4], half;
      bool win;
      rhg_band_ranges(P, pv, inv_s, B, b, r, &win, &half);
      est += (r[1] - r[0]) + (r[3] - r[2]);
    }
    if (est > kRhgHeavy) {
      if (!out) heavy[atomicAdd(nheavy, 1u)] = (uint32_t)v;
      continue;
    }
    uint64_t cnt = 0, e = out ? rp[v] : 0;
    for (int b = 0; b < P.nb; ++b) {
      uint64_t r[4], half;
      bool win;
      rhg_band_ranges(P, pv, inv_s, B, b, r, &win, &half);
      for (int part = 0; part < 2; ++part)
        for (uint64_t k = r[2 * part]; k < r[2 * part + 1]; ++k) {
          const uint32_t w = B.bl[k];
          if (!rhg_is_neighbour(P, pv, v, win, half, pt, w)) continue;
          if (out) out[e++] = (v << P.idbits) | w;
          else ++cnt;
        }
    }
    if (!out) deg[v] = (uint32_t)cnt;
  }
}

// The heavy vertices, one block each: the block's threads stride over every
// candidate range; counting adds up a block total, writing takes positions
// from a shared counter (the row order does not matter: the keys are sorted
// afterwards).
__global__ void k_rhg_heavy(rhg::Params P, RhgPts pt, RhgBands B, const uint32_t *__restrict__ heavy,
                            const unsigned int *__restrict__ nheavy, uint32_t *__restrict__ deg,
                            const uint64_t *__restrict__ rp, uint64_t *__restrict__ out) {
  __shared__ unsigned long long bcount;
  const unsigned int nh = *nheavy;
  for (unsigned int h = blockIdx.x; h < nh; h += gridDim.x) {
    const uint64_t v = heavy[h];
    const rhg::Point pv = pt.get(v);
    const double inv_s = pv.s > 0.0 ? 1.0 / pv.s : 0.0;
    if (threadIdx.x == 0) bcount = 0;
    __syncthreads();
    unsigned long long mine = 0;
    for (int b = 0; b < P.nb; ++b) {
      uint64_t r[4], half;
      bool win;
      rhg_band_ranges(P, pv, inv_s, B, b, r, &win, &half);
      for (int part = 0; part < 2; ++part)
        for (uint64_t k = r[2 * part] + threadIdx.x; k < r[2 * part + 1]; k += blockDim.x) {
          const uint32_t w = B.bl[k];
          if (!rhg_is_neighbour(P, pv, v, win, half, pt, w)) continue;
          if (out) out[rp[v] + atomicAdd(&bcount, 1ull)] = (v << P.idbits) | w;
          else ++mine;
        }
    }
    if (!out) {
      for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
      if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&bcount, mine);
    }
    __syncthreads();
    if (!out && threadIdx.x == 0) deg[v] = (uint32_t)bcount;
    __syncthreads();
  }
}

template <class T>
__global__ void k_keys_low(const uint64_t *__restrict__ keys, uint64_t nk, int b, T *__restrict__ col) {
  const uint64_t mask = (1ull << b) - 1;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nk;
       e += (uint64_t)gridDim.x * blockDim.x)
    col[e] = (T)(keys[e] & mask);
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

int cc_gen_rhg_device(cc_ctx *ctx, uint64_t n, double avg_deg, double gamma, uint64_t seed,
                      uint32_t id_bytes, uint64_t *row_ptr, void *col, uint64_t cap,
                      uint64_t *m_dir) {
  return ccg::guard([&] {
    if ((id_bytes != 4 && id_bytes != 8) || !row_ptr || !m_dir || (cap && !col))
      throw Error(CC_ERR_INVALID, "bad hyperbolic generator arguments");
    rhg::Params P;
    const int st = rhg::make_params(n, avg_deg, gamma, seed, &P);
    if (st != CC_OK) throw Error(st, "bad hyperbolic generator parameters");
    cc_ctx *C = ctx ? ctx : ccg::default_context();
    CCG_CUDA(cudaSetDevice(C->device));
    cudaStream_t s = C->stream;
    ccg::Counters c;  // with the context's profiling on, every phase is timed (cc_ctx_stats)
    c.prof = C->prof;
    c.pool = &C->ev_pool;
    const unsigned grid = ccg::grid_for(n, ccg::kBlock, ccg::num_sms() * 16);
    // points in angular order
    cudaEvent_t t0 = c.tic(s);
    DevBuf keys(8 * n, s, C->pool), tmp(8 * n, s, C->pool);
    ccg::k_rhg_keys<<<grid, ccg::kBlock, 0, s>>>(P, keys.as<uint64_t>());
    CCG_LAUNCH_CHECK();
    const uint64_t *sk = ccg::radix_sort_u64(keys.as<uint64_t>(), tmp.as<uint64_t>(), n, 64, s, C->pool, c);
    DevBuf pa(8 * n, s, C->pool), pb(8 * n, s, C->pool), ps(8 * n, s, C->pool), px(8 * n, s, C->pool),
        py(8 * n, s, C->pool), pphi(8 * n, s, C->pool), pband(4 * n, s, C->pool), bkeys(8 * n, s, C->pool);
    const ccg::RhgPts pt{pa.as<double>(), pb.as<double>(), ps.as<double>(), px.as<double>(),
                         py.as<double>(), pphi.as<uint64_t>(), pband.as<uint32_t>()};
    c.toc(s, "gen_angle_sort", t0, 0);
    t0 = c.tic(s);
    ccg::k_rhg_points<<<grid, ccg::kBlock, 0, s>>>(P, sk, pt, bkeys.as<uint64_t>());
    CCG_LAUNCH_CHECK();
    c.toc(s, "gen_points", t0, 0);
    t0 = c.tic(s);
    // vertices grouped by band, increasing id inside a band
    uint64_t *bsort = (sk == keys.as<uint64_t>()) ? tmp.as<uint64_t>() : keys.as<uint64_t>();
    int bbits = 32;
    while ((1 << (bbits - 32)) <= P.nb) ++bbits;
    const uint64_t *gk = ccg::radix_sort_u64(bkeys.as<uint64_t>(), bsort, n, bbits, s, C->pool, c);
    DevBuf bl(4 * n, s, C->pool), bstart(8 * (P.nb + 1), s, C->pool);
    ccg::k_rhg_band_starts<<<grid, ccg::kBlock, 0, s>>>(gk, n, P.nb, bstart.as<uint64_t>(),
                                                        bl.as<uint32_t>());
    CCG_LAUNCH_CHECK();
    c.toc(s, "gen_bands", t0, 0);
    std::vector<uint64_t> hb(P.nb + 1);
    CCG_CUDA(cudaMemcpyAsync(hb.data(), bstart.p, 8 * (P.nb + 1), cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    // angular cells per band
    std::vector<int> hL(P.nb);
    std::vector<uint64_t> hoff(P.nb);
    uint64_t total = 0;
    for (int b = 0; b < P.nb; ++b) {
      hL[b] = rhg::cell_bits(hb[b + 1] - hb[b]);
      hoff[b] = total;
      total += (1ull << hL[b]) + 1;
    }
    DevBuf dL(4 * P.nb, s, C->pool), doff(8 * P.nb, s, C->pool), cells(8 * total, s, C->pool);
    CCG_CUDA(cudaMemcpyAsync(dL.p, hL.data(), 4 * P.nb, cudaMemcpyHostToDevice, s));
    CCG_CUDA(cudaMemcpyAsync(doff.p, hoff.data(), 8 * P.nb, cudaMemcpyHostToDevice, s));
    const ccg::RhgBands B{bl.as<uint32_t>(), bstart.as<uint64_t>(), cells.as<uint64_t>(),
                          doff.as<uint64_t>(), dL.as<int>()};
    t0 = c.tic(s);
    ccg::k_rhg_cells<<<grid, ccg::kBlock, 0, s>>>(B, pt, gk, n, P.nb, cells.as<uint64_t>());
    CCG_LAUNCH_CHECK();
    c.toc(s, "gen_cells", t0, 0);
    keys.release();
    tmp.release();
    bkeys.release();
    // degrees, offsets, then every row's keys at its offsets
    DevBuf deg(4 * n, s, C->pool), heavy(4 * n, s, C->pool), nheavy(4, s, C->pool);
    CCG_CUDA(cudaMemsetAsync(nheavy.p, 0, 4, s));
    const unsigned hgrid = (unsigned)ccg::num_sms() * 4;
    t0 = c.tic(s);
    ccg::k_rhg_neighbours<<<grid, ccg::kBlock, 0, s>>>(P, pt, B, deg.as<uint32_t>(), nullptr, nullptr,
                                                       heavy.as<uint32_t>(), nheavy.as<unsigned int>());
    CCG_LAUNCH_CHECK();
    ccg::k_rhg_heavy<<<hgrid, ccg::kBlock, 0, s>>>(P, pt, B, heavy.as<uint32_t>(), nheavy.as<unsigned int>(),
                                                  deg.as<uint32_t>(), nullptr, nullptr);
    CCG_LAUNCH_CHECK();
    c.toc(s, "gen_count", t0, 0);
    uint64_t m = 0;
    ccg::offsets_from_counts(deg.as<uint32_t>(), n, 0, row_ptr, s, C->pool, c);
    CCG_CUDA(cudaMemcpyAsync(&m, row_ptr + n, 8, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    *m_dir = m;
    if (m >= (1ull << 32)) throw Error(CC_ERR_UNSUPPORTED, "2^32 directed entries or more");
    if (m > cap) throw Error(CC_ERR_INVALID, "col capacity below the generated entries");
    if (m == 0) return;
    DevBuf ek(8 * m, s, C->pool), et(8 * m, s, C->pool);
    t0 = c.tic(s);
    ccg::k_rhg_neighbours<<<grid, ccg::kBlock, 0, s>>>(P, pt, B, nullptr, row_ptr, ek.as<uint64_t>(),
                                                       nullptr, nullptr);
    CCG_LAUNCH_CHECK();
    ccg::k_rhg_heavy<<<hgrid, ccg::kBlock, 0, s>>>(P, pt, B, heavy.as<uint32_t>(), nheavy.as<unsigned int>(),
                                                  nullptr, row_ptr, ek.as<uint64_t>());
    CCG_LAUNCH_CHECK();
    c.toc(s, "gen_fill", t0, 0);
    // rows sorted: one sort of the (source, target) keys keeps every row in place
    t0 = c.tic(s);
    const uint64_t *sorted = ccg::radix_sort_u64(ek.as<uint64_t>(), et.as<uint64_t>(), m,
                                                 2 * P.idbits, s, C->pool, c);
    c.toc(s, "gen_row_sort", t0, 0);
    const unsigned egrid = ccg::grid_for(m, ccg::kBlock, ccg::num_sms() * 16);
    if (id_bytes == 8)
      ccg::k_keys_low<uint64_t><<<egrid, ccg::kBlock, 0, s>>>(sorted, m, P.idbits, static_cast<uint64_t *>(col));
    else
      ccg::k_keys_low<uint32_t><<<egrid, ccg::kBlock, 0, s>>>(sorted, m, P.idbits, static_cast<uint32_t *>(col));
    CCG_LAUNCH_CHECK();
    CCG_CUDA(cudaStreamSynchronize(s));
    if (c.prof) {
      cc_stats st;
      std::memset(&st, 0, sizeof(st));
      ccg::collect_kernel_stats(c, st);
      st.kernel_launches = c.launches;
      C->stats = st;
    }
  });
}

}  // extern "C"

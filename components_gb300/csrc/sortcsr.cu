// sortcsr.cu - prefix scans, a stable LSD radix sort of packed 64-bit edge keys,
// and the quotient-graph (contraction) build.
//
// The reference builds contracted graphs with hash sets and message rounds:
//   CAGBuilder::PerformLocalContraction   cag_builder.h:160-230 (unordered_set<HashedEdge>)
//   CAGBuilder::BuildLocalContractionGraph cag_builder.h:577-667 (+ ips4o sort :669-674)
//   DynamicContraction::FindExponentialConflictingEdges dynamic_contraction.h:251-290
//   DynamicContraction::InsertAndClearEdges            dynamic_contraction.h:513-559
// On one device the same quotient graph is: relabel every edge by its cluster
// ids, keep the ones whose ids differ, pack (cu, cw) into one 64-bit key,
// radix-sort, drop adjacent duplicates and rebuild the CSR.  The undirected
// dedup key of the reference (edge_hash.h:30-42, min*n+max) becomes the
// ordered pair key: both directions are kept, as the reference inserts both.
#include "kernels.h"
#include "scan.cuh"

namespace ccg {
namespace {

// ---- radix sort --------------------------------------------------------------
constexpr uint64_t kEmitPiece = 4096;  // edges per hub work item of the emit pass
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
// Keys per thread of a radix pass: 8 (2048 per block, 4 CTAs per SM at the
// scatter's registers) beat 16 (4096 per block, 2 CTAs per SM): local
// contraction's sorts 1.16 -> 0.99 ms on the 2^26 hyperbolic graph.  The
// stable digit ranks keep 16 per thread (1.09 against 1.13 ms).
constexpr int kSortItems = 8;
constexpr int kSortWarps = kBlock / 32;
constexpr int kSortTile = kBlock * kSortItems;  // 2048 keys per block
constexpr int kRankItems = 16;
constexpr int kRankTile = kBlock * kRankItems;  // 4096 digits per block

// counts[d * ntiles + tile] = keys of this tile with digit d
__global__ void k_radix_hist(const uint64_t *__restrict__ keys, uint64_t n, int shift,
                             uint32_t ntiles, uint32_t *__restrict__ counts) {
  __shared__ uint32_t h[kSortWarps][kRadix];
  for (int i = threadIdx.x; i < kSortWarps * kRadix; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  uint64_t base = (uint64_t)blockIdx.x * kSortTile + (uint64_t)w * 32 * kSortItems;
#pragma unroll 4
  for (int i = 0; i < kSortItems; ++i) {
    uint64_t idx = base + (uint64_t)i * 32 + lane;
    if (idx < n) atomicAdd(&h[w][(keys[idx] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < kSortWarps; ++k) t += h[k][d];
    counts[(uint64_t)d * ntiles + blockIdx.x] = t;
  }
}

// Stable scatter: warps own contiguous sub-tiles, lanes take consecutive keys,
// ranks inside a step come from __match_any_sync, so input order is kept for
// equal digits.
__global__ void k_radix_scatter(const uint64_t *__restrict__ keys, uint64_t *__restrict__ out,
                                uint64_t n, int shift, uint32_t ntiles,
                                const uint32_t *__restrict__ offs) {
  __shared__ uint32_t wc[kSortWarps][kRadix];
  __shared__ uint32_t gbase[kRadix];
  for (int i = threadIdx.x; i < kSortWarps * kRadix; i += blockDim.x) (&wc[0][0])[i] = 0;
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
    gbase[d] = offs[(uint64_t)d * ntiles + blockIdx.x];
  __syncthreads();
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  const unsigned lt = (1u << lane) - 1u;
  uint64_t base = (uint64_t)blockIdx.x * kSortTile + (uint64_t)w * 32 * kSortItems;
  uint64_t k[kSortItems];
  uint32_t rk[kSortItems];
#pragma unroll
  for (int i = 0; i < kSortItems; ++i) {
    uint64_t idx = base + (uint64_t)i * 32 + lane;
    bool valid = idx < n;
    k[i] = valid ? keys[idx] : 0ull;
    uint32_t d = valid ? (uint32_t)((k[i] >> shift) & (kRadix - 1)) : 0xffffu;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t before = __popc(peers & lt);
    uint32_t basecnt = (d < kRadix) ? wc[w][d] : 0u;
    __syncwarp();
    if (d < kRadix && before == 0) wc[w][d] = basecnt + __popc(peers);
    __syncwarp();
    rk[i] = (d < kRadix) ? basecnt + before : 0xffffffffu;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
    uint32_t run = 0;
#pragma unroll
    for (int q = 0; q < kSortWarps; ++q) {
      uint32_t t = wc[q][d];
      wc[q][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kSortItems; ++i) {
    if (rk[i] != 0xffffffffu) {
      uint32_t d = (uint32_t)((k[i] >> shift) & (kRadix - 1));
      out[gbase[d] + wc[w][d] + rk[i]] = k[i];
    }
  }
}

// Stable ranks of n 8-bit digits without moving anything: the same per-tile
// histograms and in-warp ranks as one radix pass, but each element writes its
// destination (rank[i], coalesced) and the inverse map (inv[pos] = i, runs of
// one digit per tile) instead of scattering keys.
__global__ void k_digit_hist(const uint8_t *__restrict__ dig, uint64_t n, uint32_t ntiles,
                             uint32_t *__restrict__ counts) {
  __shared__ uint32_t h[kSortWarps][kRadix];
  for (int i = threadIdx.x; i < kSortWarps * kRadix; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  const uint64_t base = (uint64_t)blockIdx.x * kRankTile + (uint64_t)w * 32 * kRankItems;
#pragma unroll 4
  for (int i = 0; i < kRankItems; ++i) {
    const uint64_t idx = base + (uint64_t)i * 32 + lane;
    if (idx < n) atomicAdd(&h[w][dig[idx]], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < kSortWarps; ++k) t += h[k][d];
    counts[(uint64_t)d * ntiles + blockIdx.x] = t;
  }
}
__global__ void k_digit_rank(const uint8_t *__restrict__ dig, uint64_t n, uint32_t ntiles,
                             const uint32_t *__restrict__ offs, uint32_t *__restrict__ rank,
                             uint32_t *__restrict__ inv) {
  __shared__ uint32_t wc[kSortWarps][kRadix];
  __shared__ uint32_t gbase[kRadix];
  for (int i = threadIdx.x; i < kSortWarps * kRadix; i += blockDim.x) (&wc[0][0])[i] = 0;
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
    gbase[d] = offs[(uint64_t)d * ntiles + blockIdx.x];
  __syncthreads();
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  const unsigned lt = (1u << lane) - 1u;
  const uint64_t base = (uint64_t)blockIdx.x * kRankTile + (uint64_t)w * 32 * kRankItems;
  uint32_t dg[kRankItems], rk[kRankItems];
#pragma unroll
  for (int i = 0; i < kRankItems; ++i) {
    const uint64_t idx = base + (uint64_t)i * 32 + lane;
    const uint32_t d = idx < n ? (uint32_t)dig[idx] : 0xffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t before = __popc(peers & lt);
    const uint32_t basecnt = d < kRadix ? wc[w][d] : 0u;
    __syncwarp();
    if (d < kRadix && before == 0) wc[w][d] = basecnt + __popc(peers);
    __syncwarp();
    dg[i] = d;
    rk[i] = basecnt + before;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
    uint32_t run = 0;
#pragma unroll
    for (int q = 0; q < kSortWarps; ++q) {
      const uint32_t t = wc[q][d];
      wc[q][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kRankItems; ++i) {
    if (dg[i] < kRadix) {
      const uint64_t idx = base + (uint64_t)i * 32 + lane;
      const uint32_t pos = gbase[dg[i]] + wc[w][dg[i]] + rk[i];
      rank[idx] = pos;
      inv[pos] = (uint32_t)idx;
    }
  }
}

// ---- contraction -----------------------------------------------------------

// Keys a CTA has written already: a direct-mapped set in shared memory.
// Cut edges between two clusters repeat many times on graphs with large
// components (every edge between two of them gives the same key), so dropping
// repeats before they are written shrinks the sort that follows.  A key
// replaces whatever its slot held, so the set follows the CTA's current rows
// (each CTA walks one contiguous range of rows, whose keys repeat within a few
// hundred rows) instead of filling up with the first keys it saw.  A key is
// dropped only when its slot already holds it, which means the CTA has
// written it before; a key evicted and seen again is written twice and the
// sort drops the repeat.  ~0 marks a free slot and is never a key (cluster
// ids are below n < 2^32, so both halves cannot be all ones).
constexpr uint32_t kEmitSet = 2048;  // slots (16 KB)
__device__ __forceinline__ void emit_set_clear(unsigned long long *set) {
  for (uint32_t i = threadIdx.x; i < kEmitSet; i += blockDim.x) set[i] = ~0ull;
  __syncthreads();
}
__device__ __forceinline__ bool emit_set_seen(unsigned long long *set, uint64_t key) {
  const uint32_t h = (uint32_t)mix64(key) & (kEmitSet - 1);
  if (set[h] == key) return true;  // read first: a repeat costs no atomic
  return atomicExch(set + h, (unsigned long long)key) == key;
}

// Kept keys of one warp, staged in the warp's own shared-memory buffer and
// written out with one global reservation per full buffer (one atomic per
// warp step on the single counter would serialise where keys are many).
// Repeats are dropped twice: lanes of one step holding the same key keep one
// copy (neighbouring rows of a cluster give the same key), and a buffer's keys
// pass through the CTA's set when it is written out.  Warps never wait for
// one another.
__device__ __forceinline__ uint64_t shfl_up64(uint64_t x) {
  const uint32_t lo = __shfl_up_sync(0xffffffffu, (uint32_t)x, 1);
  const uint32_t hi = __shfl_up_sync(0xffffffffu, (uint32_t)(x >> 32), 1);
  return ((uint64_t)hi << 32) | lo;
}
constexpr uint32_t kWarpKeys = 256;
constexpr unsigned kEmitCtasPerSM = 32;
constexpr uint32_t kEmitSteps = 4;  // 32-entry steps of k_emit between flush checks
constexpr uint32_t kOutList = 160;  // per warp: entries that leave their rank, resolved together
constexpr int kVecSteps = 4;        // 16-byte loads in flight per lane (virtual ranks, 32-bit ids)
struct WarpKeys {
  uint64_t *buf;
  unsigned long long *set;
  uint32_t trigger;   // flush once fill reaches this
  uint32_t fill = 0;  // warp-uniform
  __device__ __forceinline__ void flush(unsigned lane, uint64_t *__restrict__ keys,
                                        unsigned long long *__restrict__ cnt) {
    __syncwarp();
    // survivors are packed in place: chunk k0's writes land below k0 + 32, in
    // entries every lane has read already
    uint32_t out = 0;
    for (uint32_t k0 = 0; k0 < fill; k0 += 32) {
      const uint32_t k = k0 + lane;
      uint64_t key = 0;
      bool keep = false;
      if (k < fill) {
        key = buf[k];
        keep = !emit_set_seen(set, key);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) buf[out + __popc(m & ((1u << lane) - 1u))] = key;
      out += __popc(m);
    }
    __syncwarp();
    unsigned long long pos0 = 0;
    if (lane == 0 && out) pos0 = atomicAdd(cnt, (unsigned long long)out);
    pos0 = __shfl_sync(0xffffffffu, pos0, 0);
    for (uint32_t k = lane; k < out; k += 32) keys[pos0 + k] = buf[k];
    __syncwarp();
    fill = 0;
  }
  // one step of the warp, all 32 lanes: the lanes with keep set add their key,
  // except a lane whose key the lane before it also holds (lanes hold
  // consecutive entries, and neighbouring entries of a cluster's rows give
  // the same key).  The caller flushes at trigger, which leaves room for the
  // steps that come before the next check.
  __device__ __forceinline__ void put(bool keep, uint64_t key, unsigned lane) {
    const uint64_t prev = shfl_up64(key);
    const bool prev_keep = __shfl_up_sync(0xffffffffu, keep, 1);
    keep = keep && !(lane > 0 && prev_keep && prev == key);
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) buf[fill + __popc(m & ((1u << lane) - 1u))] = key;
    fill += __popc(m);
  }
};

// Emit key (cl[v] << b) | cl[w] for every kept edge (kept: the clusters differ
// and, with virtual ranks, the edge leaves v's rank; the key order does not
// matter, the sort follows).  Each warp takes 32 consecutive rows at a time
// and walks their edges as one flattened, coalesced stream (lane k reads
// entry k of the rows' concatenated adjacency; its row is the last lane whose
// degree prefix sum is <= k), so skewed degrees keep every lane busy.  Rows
// longer than hub_limit are listed as (row, piece) items for k_emit_hubs,
// which runs next on the same stream.
// RANKS: the instance for virtual ranks (rank-local row groups, their list of
// leaving entries); without ranks neither is compiled: local contraction's
// emit 5.2 -> 5.0 ms on the 2^26 hyperbolic graph (the same at five and six
// CTAs per SM).
template <class T, bool VEC, bool RANKS>
__global__ void __launch_bounds__(kBlock, VEC ? 4 : 5) k_emit(uint64_t n, const uint64_t *__restrict__ rp,
                                                 const T *__restrict__ col,
                                                 const uint32_t *__restrict__ cl, PartMap pm,
                                                 bool part, int b, uint64_t hub_limit,
                                                 uint2 *__restrict__ hub_items, uint64_t hub_cap,
                                                 unsigned int *__restrict__ n_hub_items,
                                                 uint64_t *__restrict__ keys,
                                                 unsigned long long *__restrict__ cnt,
                                                 uint64_t m) {
  __shared__ uint64_t wbuf[kBlock / 32][kWarpKeys];
  __shared__ uint64_t wout[RANKS ? kBlock / 32 : 1][RANKS ? kOutList : 1];
  __shared__ unsigned long long set[kEmitSet];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  emit_set_clear(set);
  WarpKeys st{wbuf[wid], set, kWarpKeys - 32 * kEmitSteps};
  uint64_t *olist = wout[RANKS ? wid : 0];
  // the CTA's rows: one contiguous range (a multiple of 32 rows), so that the
  // keys its set holds are those of its current rows
  const uint64_t per = ((n + gridDim.x - 1) / gridDim.x + 31) / 32 * 32;
  const uint64_t r1 = min(n, (blockIdx.x + 1) * per);
  // each group's row offsets are loaded while the group before it is walked
  uint64_t next_b = 0, next_e = 0;
  if (blockIdx.x * per + 32 * wid + lane < n) {
    next_b = __ldg(rp + blockIdx.x * per + 32 * wid + lane);
    next_e = __ldg(rp + blockIdx.x * per + 32 * wid + lane + 1);
  }
  for (uint64_t v0 = blockIdx.x * per + 32 * wid; v0 < r1; v0 += blockDim.x) {
    const uint64_t v = v0 + lane;
    uint64_t eb = 0;
    uint32_t deg = 0, lo = 0, hi = 0xffffffffu;  // lo, hi: v's rank when part
    bool hub = false;
    const uint64_t cur_b = next_b, cur_e = next_e;
    if (v0 + blockDim.x < r1 && v + blockDim.x < n) {
      next_b = __ldg(rp + v + blockDim.x);
      next_e = __ldg(rp + v + blockDim.x + 1);
    }
    if (v < n) {
      eb = cur_b;
      const uint64_t ee = cur_e;
      if (ee - eb <= hub_limit) {
        deg = (uint32_t)(ee - eb);
      } else {
        // a long row becomes ceil(d / kEmitPiece) warp-sized work items
        hub = true;
        const uint32_t np = (uint32_t)((ee - eb + kEmitPiece - 1) / kEmitPiece);
        const unsigned int slot = atomicAdd(n_hub_items, np);
        for (uint32_t q = 0; q < np && (uint64_t)slot + q < hub_cap; ++q)
          hub_items[slot + q] = make_uint2((uint32_t)v, q);
      }
      if (part) pm.bounds((uint32_t)v, lo, hi);
    }
    uint32_t inc = deg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if ((int)lane >= o) inc += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    const uint32_t off = inc - deg;
    constexpr int kSteps = (int)kEmitSteps;
    // Virtual ranks, the 32 rows in one rank and none of them a hub row (the
    // common case): the rows' entries are one contiguous range, and an entry
    // is kept only if it leaves the rank, which needs no row.  Each step
    // loads and tests 32 entries; only a step that keeps some (a few in a
    // hundred on the hyperbolic graph) finds the rows of its entries.
    const uint32_t lo0 = __shfl_sync(0xffffffffu, lo, 0), hi0 = __shfl_sync(0xffffffffu, hi, 0);
    if (RANKS && part && !__any_sync(0xffffffffu, hub || (v < n && (lo != lo0 || hi != hi0)))) {
      const uint64_t base = ((uint64_t)__shfl_sync(0xffffffffu, (uint32_t)(eb >> 32), 0) << 32) |
                            __shfl_sync(0xffffffffu, (uint32_t)eb, 0);
      // entries that leave the rank are listed as (offset, id) and resolved
      // together (row search, both clusters, key) once per group, so that the
      // group waits for one round of gathers instead of one per step
      uint32_t on = 0;  // warp-uniform
      auto drain = [&]() {
        __syncwarp();
        for (uint32_t k0 = 0; k0 < on; k0 += 32) {
          const bool have = k0 + lane < on;
          const uint64_t e = have ? olist[k0 + lane] : 0ull;
          const uint32_t ff = (uint32_t)(e >> 32), u = (uint32_t)e;
          int r = 0;
#pragma unroll
          for (int step = 16; step; step >>= 1) {
            const uint32_t o = __shfl_sync(0xffffffffu, off, r + step);
            if (o <= ff) r += step;
          }
          bool keep = false;
          uint64_t key = 0;
          if (have) {
            const uint32_t cvr = cl[v0 + r], cu = cl[u];
            key = ((uint64_t)cvr << b) | cu;
            keep = cu != cvr;
          }
          st.put(keep, key, lane);
          if (st.fill >= st.trigger) st.flush(lane, keys, cnt);
        }
        __syncwarp();
        on = 0;
      };
      if constexpr (VEC && sizeof(T) == 4) {
        // 16-byte loads: lane j of a step reads entries a0 + 4j .. a0 + 4j + 3
        // (a0 = the group's first entry rounded down to a multiple of four),
        // kVecSteps such loads per lane in flight together, which covers a
        // typical 32-row group at once.  Entries outside the group are
        // loaded and ignored; a vector that would reach past the id array is
        // read entry by entry.
        const uint64_t a0 = base & ~3ull;
        const uint32_t head = (uint32_t)(base - a0);
        const uint32_t nv = (head + total + 3) / 4;
        for (uint32_t j0 = 0; j0 < nv; j0 += 32 * kVecSteps) {
          uint4 w[kVecSteps];
#pragma unroll
          for (int q = 0; q < kVecSteps; ++q) {
            const uint32_t j = j0 + 32 * q + lane;
            const uint64_t e = a0 + 4ull * j;
            w[q] = make_uint4(lo0, lo0, lo0, lo0);  // inside the rank: never kept
            if (j < nv) {
              if (e + 4 <= m) {
                w[q] = __ldg(reinterpret_cast<const uint4 *>(col + e));
              } else {
                if (e < m) w[q].x = (uint32_t)col[e];
                if (e + 1 < m) w[q].y = (uint32_t)col[e + 1];
                if (e + 2 < m) w[q].z = (uint32_t)col[e + 2];
              }
            }
          }
#pragma unroll
          for (int q = 0; q < kVecSteps; ++q) {
            if (j0 + 32 * q >= nv) continue;  // warp-uniform
            if (on > kOutList - 128) drain();  // room for this vector's entries
            const uint32_t f4 = 4 * (j0 + 32 * q + lane);  // f of component 0, plus head
            const uint32_t uu[4] = {w[q].x, w[q].y, w[q].z, w[q].w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const uint32_t u = uu[t];
              const bool in_group = f4 + t >= head && f4 + t - head < total;
              const bool out = in_group && (u < lo0 || u >= hi0);
              const unsigned om = __ballot_sync(0xffffffffu, out);
              if (out)
                olist[on + __popc(om & ((1u << lane) - 1u))] =
                    ((uint64_t)(f4 + t - head) << 32) | u;
              on += __popc(om);
            }
          }
        }
      } else {
        for (uint32_t f0 = 0; f0 < total; f0 += 32 * kSteps) {
          uint32_t us[kSteps];
#pragma unroll
          for (int q = 0; q < kSteps; ++q) {
            const uint32_t f = f0 + 32 * q + lane;
            us[q] = f < total ? load_id(col, base + f) : lo0;  // past the range: inside the rank
          }
#pragma unroll
          for (int q = 0; q < kSteps; ++q) {
            const uint32_t u = us[q];
            const bool out = u < lo0 || u >= hi0;  // false past the range
            const unsigned om = __ballot_sync(0xffffffffu, out);
            if (out)
              olist[on + __popc(om & ((1u << lane) - 1u))] = ((uint64_t)(f0 + 32 * q + lane) << 32) | u;
            on += __popc(om);
          }
          if (on > kOutList - 32 * kSteps) drain();  // room for the next batch
        }
      }
      if (on) drain();
      continue;
    }
    const uint32_t cv = v < n ? cl[v] : 0u;
    // four steps of 32 entries at a time: their loads are issued together
    // (one load in flight per warp left the pass latency-bound)
    for (uint32_t f0 = 0; f0 < total; f0 += 32 * kSteps) {
      uint32_t us[kSteps];
      int rs[kSteps];
#pragma unroll
      for (int q = 0; q < kSteps; ++q) {
        const uint32_t f = f0 + 32 * q + lane;
        int r = 0;
#pragma unroll
        for (int step = 16; step; step >>= 1) {
          const uint32_t o = __shfl_sync(0xffffffffu, off, r + step);
          if (o <= f) r += step;
        }
        rs[q] = r;
        const uint32_t ro = __shfl_sync(0xffffffffu, off, r);
        const uint64_t ebr = ((uint64_t)__shfl_sync(0xffffffffu, (uint32_t)(eb >> 32), r) << 32) |
                             __shfl_sync(0xffffffffu, (uint32_t)eb, r);
        us[q] = f < total ? load_id(col, ebr + (f - ro)) : 0u;
      }
#pragma unroll
      for (int q = 0; q < kSteps; ++q) {
        if (f0 + 32 * q >= total) break;  // warp-uniform
        const int r = rs[q];
        const uint32_t u = us[q];
        const uint32_t cvr = __shfl_sync(0xffffffffu, cv, r);
        const uint32_t lor = __shfl_sync(0xffffffffu, lo, r);
        const uint32_t hir = __shfl_sync(0xffffffffu, hi, r);
        bool keep = false;
        uint64_t key = 0;
        if (f0 + 32 * q + lane < total && (!part || u < lor || u >= hir)) {
          const uint32_t cu = cl[u];  // no gather for edges inside a rank
          key = ((uint64_t)cvr << b) | cu;
          keep = cu != cvr;
        }
        st.put(keep, key, lane);
      }
      if (st.fill >= st.trigger) st.flush(lane, keys, cnt);
    }
  }
  if (st.fill) st.flush(lane, keys, cnt);
}

// One warp per piece of a hub row (rows longer than the k_emit limit):
// kEmitPiece edges each, so the longest row is spread over many warps.
template <class T>
__global__ void __launch_bounds__(kBlock) k_emit_hubs(
    const uint64_t *__restrict__ rp, const T *__restrict__ col, const uint32_t *__restrict__ cl,
    PartMap pm, bool part, int b, const uint2 *__restrict__ items, uint64_t cap,
    const unsigned int *__restrict__ d_nitems, uint64_t *__restrict__ keys,
    unsigned long long *__restrict__ cnt) {
  __shared__ uint64_t wbuf[kBlock / 32][kWarpKeys];
  __shared__ unsigned long long set[kEmitSet];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  emit_set_clear(set);
  WarpKeys st{wbuf[wid], set, kWarpKeys - 32};
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t nitems = min((uint64_t)*d_nitems, cap);
  for (uint64_t h = warp; h < nitems; h += nwarps) {
    const uint2 it = items[h];
    const uint32_t v = it.x;
    const uint64_t re = __ldg(rp + v + 1);
    const uint64_t eb = __ldg(rp + v) + (uint64_t)it.y * kEmitPiece;
    const uint64_t ee = min(re, eb + kEmitPiece);
    const uint32_t cv = cl[v];
    uint32_t lo = 0, hi = 0xffffffffu;  // v's rank when part
    if (part) pm.bounds(v, lo, hi);
    // four steps of 32 entries at a time: their id loads are issued together,
    // then the cluster gathers of the entries that can be kept (with virtual
    // ranks only those that leave the rank: most entries of a hub row stay
    // inside it)
    constexpr int kSteps = (int)kEmitSteps;
    for (uint64_t e0 = eb; e0 < ee; e0 += 32 * kSteps) {
      uint32_t us[kSteps], cus[kSteps];
#pragma unroll
      for (int q = 0; q < kSteps; ++q) {
        const uint64_t e = e0 + 32 * q + lane;
        us[q] = e < ee ? load_id(col, e) : 0u;
      }
#pragma unroll
      for (int q = 0; q < kSteps; ++q) {
        const uint64_t e = e0 + 32 * q + lane;
        const bool need = e < ee && (!part || us[q] < lo || us[q] >= hi);
        cus[q] = need ? cl[us[q]] : cv;  // cv: not kept
      }
#pragma unroll
      for (int q = 0; q < kSteps; ++q) {
        st.put(cus[q] != cv, ((uint64_t)cv << b) | cus[q], lane);
        if (st.fill >= st.trigger) st.flush(lane, keys, cnt);
      }
    }
  }
  if (st.fill) st.flush(lane, keys, cnt);
}

struct GetUniq {
  const uint64_t *k;
  __device__ uint32_t operator()(uint64_t i) const { return (i == 0 || k[i] != k[i - 1]) ? 1u : 0u; }
};
struct PutUniq {
  const uint64_t *k;
  uint64_t *o;
  __device__ void operator()(uint64_t i, uint32_t excl, uint32_t f) const {
    if (f) o[excl] = k[i];
  }
};
// New vertex ids of the component graph: the sources of the unique keys in
// key order (the sorted keys of one source are adjacent), numbered by a scan
// over the unique keys.  The first key of each source also gives that
// vertex's row start and its original id.  Clusters with no key keep kNone
// (set before the scan).
struct GetSrcStart {
  const uint64_t *uk;
  const uint32_t *d_u;  // number of unique keys
  int b;
  __device__ uint32_t operator()(uint64_t i) const {
    if (i >= *d_u) return 0u;
    return (i == 0 || (uk[i] >> b) != (uk[i - 1] >> b)) ? 1u : 0u;
  }
};
struct PutSrcId {
  const uint64_t *uk;
  int b;
  uint32_t *newid, *vid;
  uint64_t *rp;
  const uint32_t *vid_of_cluster;  // null: a cluster's id is its original id
  __device__ void operator()(uint64_t i, uint32_t excl, uint32_t f) const {
    if (!f) return;
    const uint32_t c = (uint32_t)(uk[i] >> b);
    newid[c] = excl;
    vid[excl] = vid_of_cluster ? vid_of_cluster[c] : c;
    rp[excl] = i;
  }
};

__global__ void k_build_csr(const uint64_t *__restrict__ uk, const uint32_t *__restrict__ d_u,
                            int b, const uint32_t *__restrict__ newid, uint64_t *__restrict__ rp,
                            uint32_t *__restrict__ col, const uint32_t *__restrict__ d_nv) {
  uint32_t u = *d_u;
  const uint64_t mask = (b == 64) ? ~0ull : ((1ull << b) - 1);
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < u;
       e += (uint64_t)gridDim.x * blockDim.x)
    col[e] = newid[(uint32_t)(uk[e] & mask)];
  if (blockIdx.x == 0 && threadIdx.x == 0) rp[*d_nv] = u;
}

int bits_for(uint64_t x) {  // bits needed to hold values < x
  int b = 1;
  while (b < 64 && (1ull << b) < x) ++b;
  return b;
}

template <class T>
void emit_keys(const Csr &g, const uint32_t *cl, const PartMap &pm, bool part, int b,
               uint64_t *keys, unsigned long long *cnt, cudaStream_t s, cudaMemPool_t pool,
               Counters &c) {
  const T *col = static_cast<const T *>(g.col);
  // k_emit streams rows up to hub_limit entries; longer rows go to the
  // piece-per-warp kernel so that one hub does not hold one warp for long.
  // (One thread per row, with the repeats dropped in a warp buffer and the
  // CTA's set, was measured slower without virtual ranks: 7.5 ms against
  // 5.3 ms for local contraction's first level on the 2^26-vertex hyperbolic
  // graph.)
  // With virtual ranks most row groups take the rank-local stream, which
  // suits longer rows: the 16-rank emit on the 2^26-vertex hyperbolic graph
  // took 2.14 / 1.91 / 1.80 / 1.85 / 2.04 ms with limits of 256 / 1024 / 4096
  // / 16384 / 65536 entries; without ranks 1024 beats 4096 (5.22 against
  // 5.44 ms over local contraction's levels).
  const uint64_t hub_limit = part ? 4096 : 1024;
  const uint64_t cap = g.m / (hub_limit + 1) + g.m / kEmitPiece + 2;
  DevBuf hubs(8 * cap, s, pool), nh(4, s, pool);
  CCG_CUDA(cudaMemsetAsync(nh.p, 0, 4, s));
  const unsigned egrid = grid_for(g.n, kBlock, num_sms() * kEmitCtasPerSM);
  cudaEvent_t t0 = c.tic(s);
  // virtual ranks, 32-bit ids on a 16-byte aligned array: the rank-local
  // groups stream their entries with 16-byte loads
  if (part && sizeof(T) == 4 && (reinterpret_cast<uintptr_t>(col) & 15) == 0)
    k_emit<T, true, true><<<egrid, kBlock, 0, s>>>(g.n, g.rp, col, cl, pm, part, b, hub_limit,
                                                   hubs.as<uint2>(), cap, nh.as<unsigned int>(), keys,
                                                   cnt, g.m);
  else if (part)
    k_emit<T, false, true><<<egrid, kBlock, 0, s>>>(g.n, g.rp, col, cl, pm, part, b, hub_limit,
                                                    hubs.as<uint2>(), cap, nh.as<unsigned int>(), keys,
                                                    cnt, g.m);
  else
    k_emit<T, false, false><<<egrid, kBlock, 0, s>>>(g.n, g.rp, col, cl, pm, part, b, hub_limit,
                                                     hubs.as<uint2>(), cap, nh.as<unsigned int>(),
                                                     keys, cnt, g.m);
  CCG_LAUNCH_CHECK();
  // at most cap pieces, one warp each: a small graph gets a small grid (every
  // CTA clears its 16 KB key set, which had cost 45 us per launch on the
  // small level graphs of local contraction)
  const unsigned hgrid = (unsigned)std::min<uint64_t>((uint64_t)num_sms() * kEmitCtasPerSM,
                                                      (cap + kBlock / 32 - 1) / (kBlock / 32));
  k_emit_hubs<T><<<hgrid, kBlock, 0, s>>>(
      g.rp, col, cl, pm, part, b, hubs.as<uint2>(), cap, nh.as<unsigned int>(), keys, cnt);
  CCG_LAUNCH_CHECK();
  // algorithmic bytes: offsets, ids and own clusters; a neighbour's cluster
  // is gathered per entry without virtual ranks, and with them only for the
  // entries that leave their rank (about one in a hundred, not counted)
  c.toc(s, "contract_emit", t0,
        8 * (g.n + 1) + g.m * ((uint64_t)g.idb + (part ? 0 : 4)) + 4 * g.n);
  // relabel + compact: offsets, neighbour id and its cluster per edge, own
  // cluster per vertex (the emitted keys are counted at the sort)
  c.add(3, 8 * (g.n + 1) + g.m * ((uint64_t)g.idb + 4) + 4 * g.n);
}

}  // namespace

namespace {
struct GetDeg {
  const uint8_t *d;
  __device__ uint32_t operator()(uint64_t i) const { return d[i]; }
};
struct GetCount {
  const uint32_t *d;
  __device__ uint32_t operator()(uint64_t i) const { return d[i]; }
};
// Degree bytes with escapes: byte 255 stands for the exact degree held by the
// (row, degree) pair of that row in esc (sorted by row).
struct GetDegEsc {
  const uint8_t *d;
  const uint2 *esc;
  uint32_t nesc;
  uint32_t first_row;
  __device__ uint32_t operator()(uint64_t i) const {
    const uint32_t x = d[i];
    if (x != 255) return x;
    const uint32_t row = first_row + (uint32_t)i;
    uint32_t lo = 0, hi = nesc;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (esc[mid].x < row) lo = mid + 1;
      else hi = mid;
    }
    return lo < nesc ? esc[lo].y : 0u;
  }
};
struct PutOffset {
  uint64_t *rp;
  uint64_t base;
  __device__ void operator()(uint64_t i, uint32_t excl, uint32_t f) const {
    rp[i + 1] = base + excl + f;
    if (i == 0) rp[0] = base;
  }
};
}  // namespace

namespace {
struct GetNonzero {
  const uint32_t *h;
  __device__ uint32_t operator()(uint64_t i) const { return h[i] ? 1u : 0u; }
};
struct PutPair {
  const uint32_t *h;
  uint64_t *pairs;
  uint64_t cap;
  __device__ void operator()(uint64_t i, uint32_t excl, uint32_t f) const {
    if (f && excl < cap) {
      pairs[2 * (uint64_t)excl] = i;
      pairs[2 * (uint64_t)excl + 1] = h[i];
    }
  }
};
}  // namespace

void compact_histogram(const uint32_t *hist, uint64_t len, uint64_t *pairs, uint64_t cap,
                       uint32_t *d_count, cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  scan_generic(len, GetNonzero{hist}, PutPair{hist, pairs, cap}, d_count, s, pool, c);
}

void unique_sorted_keys(const uint64_t *sorted, uint64_t n, uint64_t *out, uint32_t *d_count,
                        cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  scan_generic(n, GetUniq{sorted}, PutUniq{sorted, out}, d_count, s, pool, c);
}

void offsets_from_degrees(const uint8_t *deg, uint64_t count, uint64_t base, uint64_t *rp,
                          cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  if (count == 0) return;
  scan_generic(count, GetDeg{deg}, PutOffset{rp, base}, nullptr, s, pool, c);
}

void offsets_from_degrees_esc(const uint8_t *deg, uint64_t count, uint64_t first_row, uint64_t base,
                              const uint2 *esc, uint32_t nesc, uint64_t *rp, cudaStream_t s,
                              cudaMemPool_t pool, Counters &c) {
  if (count == 0) return;
  scan_generic(count, GetDegEsc{deg, esc, nesc, (uint32_t)first_row}, PutOffset{rp, base}, nullptr, s,
               pool, c);
}

void offsets_from_counts(const uint32_t *deg, uint64_t count, uint64_t base, uint64_t *rp,
                         cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  if (count == 0) return;
  scan_generic(count, GetCount{deg}, PutOffset{rp, base}, nullptr, s, pool, c);
}

void stable_digit_ranks(const uint8_t *dig, uint64_t n, uint32_t *rank, uint32_t *inv,
                        cudaStream_t s, cudaMemPool_t pool, Counters &c) {
  if (n == 0) return;
  if (n >= (1ull << 32)) throw Error(CC_ERR_UNSUPPORTED, "digit ranks: more than 2^32 elements");
  const uint32_t ntiles = (uint32_t)((n + kRankTile - 1) / kRankTile);
  DevBuf counts(4ull * kRadix * ntiles, s, pool);
  k_digit_hist<<<ntiles, kBlock, 0, s>>>(dig, n, ntiles, counts.as<uint32_t>());
  CCG_LAUNCH_CHECK();
  scan_generic((uint64_t)kRadix * ntiles, GetArr{counts.as<uint32_t>()},
               PutArr{counts.as<uint32_t>()}, nullptr, s, pool, c);
  k_digit_rank<<<ntiles, kBlock, 0, s>>>(dig, n, ntiles, counts.as<uint32_t>(), rank, inv);
  CCG_LAUNCH_CHECK();
  c.add(2, 2 * n + 8 * n);
}

uint64_t *radix_sort_u64(uint64_t *keys, uint64_t *tmp, uint64_t n, int bits, cudaStream_t s,
                         cudaMemPool_t pool, Counters &c) {
  if (n <= 1) return keys;
  if (n >= (1ull << 32)) throw Error(CC_ERR_UNSUPPORTED, "radix sort: more than 2^32 keys");
  uint32_t ntiles = (uint32_t)((n + kSortTile - 1) / kSortTile);
  DevBuf counts(4ull * kRadix * ntiles, s, pool);
  uint64_t *src = keys, *dst = tmp;
  for (int shift = 0; shift < bits; shift += kRadixBits) {
    k_radix_hist<<<ntiles, kBlock, 0, s>>>(src, n, shift, ntiles, counts.as<uint32_t>());
    CCG_LAUNCH_CHECK();
    scan_generic((uint64_t)kRadix * ntiles, GetArr{counts.as<uint32_t>()},
                 PutArr{counts.as<uint32_t>()}, nullptr, s, pool, c);
    k_radix_scatter<<<ntiles, kBlock, 0, s>>>(src, dst, n, shift, ntiles, counts.as<uint32_t>());
    CCG_LAUNCH_CHECK();
    c.add(2, 8 * n * 3);  // hist read + scatter read + write
    uint64_t *t = src;
    src = dst;
    dst = t;
  }
  return src;
}

void contract_graph(const Csr &g, const uint32_t *cl, uint64_t ncl,
                    const uint32_t *vid_of_cluster, const PartMap *pm, Contracted &out,
                    cudaStream_t s, cudaMemPool_t pool, Counters &c, uint32_t *host_mailbox) {
  out = Contracted();
  out.newid.alloc(4 * (ncl ? ncl : 1), s, pool);
  if (g.m == 0 || g.n == 0) {
    CCG_CUDA(cudaMemsetAsync(out.newid.p, 0xff, 4 * ncl, s));
    out.rp.alloc(8, s, pool);
    CCG_CUDA(cudaMemsetAsync(out.rp.p, 0, 8, s));
    return;
  }
  if (ncl >= (1ull << 32) - 1) throw Error(CC_ERR_UNSUPPORTED, "contract: too many clusters");
  const int b = bits_for(ncl);
  PartMap p = pm ? *pm : PartMap(g.n, 1);
  DevBuf keys(8 * g.m, s, pool);
  DevBuf cnt(8, s, pool);
  CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 8, s));
  if (g.idb == 8)
    emit_keys<uint64_t>(g, cl, p, pm != nullptr, b, keys.as<uint64_t>(),
                        cnt.as<unsigned long long>(), s, pool, c);
  else
    emit_keys<uint32_t>(g, cl, p, pm != nullptr, b, keys.as<uint64_t>(),
                        cnt.as<unsigned long long>(), s, pool, c);
  unsigned long long ne = 0;
  CCG_CUDA(cudaMemcpyAsync(&ne, cnt.p, 8, cudaMemcpyDeviceToHost, s));
  CCG_CUDA(cudaStreamSynchronize(s));
  (void)host_mailbox;
  if (ne == 0) {
    CCG_CUDA(cudaMemsetAsync(out.newid.p, 0xff, 4 * ncl, s));
    out.rp.alloc(8, s, pool);
    CCG_CUDA(cudaMemsetAsync(out.rp.p, 0, 8, s));
    return;
  }
  DevBuf tmp(8 * ne, s, pool);
  cudaEvent_t ts = c.tic(s);
  uint64_t *sorted = radix_sort_u64(keys.as<uint64_t>(), tmp.as<uint64_t>(), ne, 2 * b, s, pool, c);
  c.toc(s, "contract_sort", ts, 24 * ne * (uint64_t)((2 * b + 7) / 8));
  cudaEvent_t td = c.tic(s);
  // unique keys into the other buffer
  uint64_t *uk = (sorted == keys.as<uint64_t>()) ? tmp.as<uint64_t>() : keys.as<uint64_t>();
  DevBuf d_u(4, s, pool), d_nv(4, s, pool);
  scan_generic(ne, GetUniq{sorted}, PutUniq{sorted, uk}, d_u.as<uint32_t>(), s, pool, c);
  c.add(0, 8 * ne + 8 * ne);  // dedup: read keys, write uniques (upper bound)
  // new ids (order preserving), original ids and row starts from the unique
  // keys alone: no pass over all ncl clusters but the kNone fill.  Every new
  // vertex is the source of a unique key, so ne bounds their number.
  CCG_CUDA(cudaMemsetAsync(out.newid.p, 0xff, 4 * ncl, s));
  out.rp.alloc(8 * (ne + 1), s, pool);
  out.vid.alloc(4 * ne, s, pool);
  scan_generic(ne, GetSrcStart{uk, d_u.as<uint32_t>(), b},
               PutSrcId{uk, b, out.newid.as<uint32_t>(), out.vid.as<uint32_t>(), out.rp.as<uint64_t>(),
                        vid_of_cluster},
               d_nv.as<uint32_t>(), s, pool, c);
  c.toc(s, "contract_dedup", td, 16 * ne + 4 * ncl + 8 * ne);
  uint32_t uv[2];
  CCG_CUDA(cudaMemcpyAsync(&uv[0], d_u.p, 4, cudaMemcpyDeviceToHost, s));
  CCG_CUDA(cudaMemcpyAsync(&uv[1], d_nv.p, 4, cudaMemcpyDeviceToHost, s));
  CCG_CUDA(cudaStreamSynchronize(s));
  out.m = uv[0];
  out.n = uv[1];
  out.col.alloc(4 * out.m, s, pool);
  cudaEvent_t tb = c.tic(s);
  k_build_csr<<<grid_for(out.m, kBlock, num_sms() * 16), kBlock, 0, s>>>(
      uk, d_u.as<uint32_t>(), b, out.newid.as<uint32_t>(), out.rp.as<uint64_t>(),
      out.col.as<uint32_t>(), d_nv.as<uint32_t>());
  CCG_LAUNCH_CHECK();
  // CSR rebuild: unique keys read, ids written, one target id gathered each
  c.toc(s, "contract_csr", tb, 8 * out.m + 4 * out.m + 4 * out.m);
  c.add(2, 16 * out.m + 4 * ncl + 8 * ne);
}

}  // namespace ccg

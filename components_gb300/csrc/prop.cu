// prop.cu - label propagation, shortcut (pointer-jumping) propagation, label
// composition and canonicalisation.
#include "kernels.h"

namespace ccg {
// Shortcut and label rounds bound to eight CTAs of 256 threads per SM (32
// registers): the in-place label round had taken 34-40 registers, six CTAs
// per SM, and these latency-bound gathers run faster with the two extra CTAs
// (label propagation on the 2^26 hyperbolic graph: 18.2 -> 16.9 ms).
constexpr int kSweepCtasPerSM = 8;
namespace {

// Rows above a limit are relaxed a warp per piece of 2048 entries (the
// *_pieces kernels); shorter rows a thread each.  On the 2^26-vertex
// hyperbolic graph the best limit differs per option: label propagation
// 25.7 / 19.2 / 18.1 ms and shortcuts 13.2 / 13.0 / 13.9 ms for limits of
// 64 / 128 / 256 entries.
// A round visits only the rows next to the labels changed in the round before
// once at most V / div labels changed: label propagation 16.9 / 16.3 ms with
// div 16 / 2 (33.8 ms with div 1: every round through the neighbour marks)
// and shortcuts 13.1 / 11.8 ms with div 16 / 8 (div 4 and 2 the same) on the
// 2^26-vertex hyperbolic graph.
constexpr uint64_t kLabelSparseDiv = 2, kShortcutSparseDiv = 8;
constexpr uint64_t kLabelRowLimit = 256, kShortcutRowLimit = 128;

// ---- Propagation (propagation.h:72-149) ------------------------------------
// lab[v] <- min(lab[v], min_u lab[u]) in place.  The reference updates local
// vertices in place during a sweep (SetVertexPayload) and sees ghosts from
// the last exchange; on one device every vertex is local.
// A lowered label sets its vertex's bit in chg and is counted (one atomic per
// block into *nchanged).  act (null: every row) marks the rows to visit: the
// neighbours of the labels lowered in the round before.  A row left out then
// already sits at or below every neighbour's label: a neighbour whose label
// last changed in round k is in round k's changed set, so the row is visited
// in round k + 1 after that change; when a round changes no label, every row
// is at its neighbours' minimum, as after a round over every row.
__device__ __forceinline__ bool bit_of(const uint32_t *bits, uint64_t v) {
  return (bits[v >> 5] >> (v & 31)) & 1u;
}
// CHECK (the first round over a caller's ids that no pass has checked): an
// id >= n is skipped and recorded in *err; the host reads *err after the round
// and stops before any kernel trusts the ids.
template <bool CHECK>
__global__ void __launch_bounds__(kBlock, kSweepCtasPerSM) k_labels_round(uint64_t n, const uint64_t *__restrict__ rp,
                               const uint32_t *__restrict__ col, uint32_t *lab,
                               const uint32_t *__restrict__ act, uint32_t *__restrict__ chg,
                               unsigned int *nchanged, int *err, uint64_t row_limit) {
  __shared__ unsigned int block_changed;
  if (threadIdx.x == 0) block_changed = 0;
  __syncthreads();
  const uint64_t span = (n + 31) / 32 * 32;  // warp-uniform trip count, 32-aligned lanes
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < span;
       v += (uint64_t)gridDim.x * blockDim.x) {
    bool changed = false;
    if (v < n && (!act || bit_of(act, v))) {
      const uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
      if (e - b <= row_limit) {
        const uint32_t l = ld_cg(lab + v);
        bool bad = false;
        const uint32_t best = row_min_ilp<uint32_t>(col, b, e, l, [&](uint32_t u) {
          if (CHECK && u >= n) {
            bad = true;
            return kNone;
          }
          return ld_cg(lab + u);
        });
        if (CHECK && bad) set_err(err, kErrBadId);
        if (best < l) {
          st_cg(lab + v, best);
          changed = true;
        }
      }
    }
    const unsigned bm = __ballot_sync(0xffffffffu, changed);
    if ((threadIdx.x & 31) == 0 && bm) {
      chg[v >> 5] = bm;  // the warp's own word (chg is cleared before the round)
      atomicAdd(&block_changed, (unsigned)__popc(bm));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && block_changed) atomicAdd(nchanged, block_changed);
}

// Rows above the row limit, one warp per piece of the row.
template <bool CHECK>
__global__ void k_labels_round_pieces(uint64_t n, const uint64_t *__restrict__ rp,
                                      const uint32_t *__restrict__ col, RowPieces rpc, uint32_t *lab,
                                      const uint32_t *__restrict__ act, uint32_t *chg,
                                      unsigned int *nchanged, int *err) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t ni = min((uint64_t)*rpc.count, rpc.cap);
  for (uint64_t h = warp; h < ni; h += nwarps) {
    uint32_t v;
    uint64_t b, e;
    row_piece(rpc, rp, h, v, b, e);
    if (act && !bit_of(act, v)) continue;  // warp-uniform: one row per piece
    bool bad = false;
    uint32_t best = piece_min_ilp<uint32_t>(col, b, e, lane, kNone, [&](uint32_t u) {
      if (CHECK && u >= n) {
        bad = true;
        return kNone;
      }
      return ld_cg(lab + u);
    });
    if (CHECK && bad) set_err(err, kErrBadId);
    best = __reduce_min_sync(0xffffffffu, best);
    if (lane == 0 && best < ld_cg(lab + v)) {
      atomicMin(lab + v, best);
      atomicOr(chg + (v >> 5), 1u << (v & 31));
      atomicAdd(nchanged, 1u);  // a row of several pieces may count more than once
    }
  }
}

// ---- ShortcutPropagation (shortcut_propagation.h:124-376) ------------------
// Round, with f = current labels (g labels) and nf = labels_:
//   FindMinLabels (:194-208):  nf[v] = min over N[v] of f
//   Shortcut      (:225-357):  an update (f[v] -> nf[v]) for every v whose
//                              label drops; a request for f[nf[v]]; both
//                              answers are applied to every u with nf[u]
//                              equal to the target
//   CheckConvergence (:359-376): stop when nf == f everywhere.
// The update to label l is the minimum over the rows labelled l.  From the
// second round on most rows share a few labels (a hundred thousand rows per
// label on a 2^20-vertex hyperbolic graph), so the updates go through
// warp_min_to: one atomic per distinct label in a warp, none when the entry
// already holds as little.
// act (null: every row) marks the rows with a neighbour whose label changed
// in the previous round.  A row without one keeps its label and sends no
// update: its neighbours' minimum m is the previous round's, that round set
// nf[v] <= m, and the jump only lowered it, so min(f[v], m) = f[v].
// CHECK: as in k_labels_round.
template <bool CHECK>
__global__ void __launch_bounds__(kBlock, kSweepCtasPerSM) k_sc_min(uint64_t n, const uint64_t *__restrict__ rp,
                         const uint32_t *__restrict__ col, const uint32_t *__restrict__ f,
                         uint32_t *__restrict__ nf, uint32_t *upd,
                         const uint32_t *__restrict__ act, int *err, uint64_t row_limit) {
  const uint64_t span = (n + 31) / 32 * 32;  // warp-uniform trip count
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < span;
       v += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t l = 0, best = 0;
    if (v < n) {
      l = f[v];
      best = l;
      if (!act || bit_of(act, v)) {
        const uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
        bool bad = false;
        if (e - b <= row_limit)  // longer rows: k_sc_min_pieces folds their neighbours in
          best = row_min_ilp<uint32_t>(col, b, e, l, [&](uint32_t u) {
            if (CHECK && u >= n) {
              bad = true;
              return kNone;
            }
            return __ldg(f + u);
          });
        if (CHECK && bad) set_err(err, kErrBadId);
      }
      nf[v] = best;
    }
    warp_min_to(upd, best < l, l, best);
  }
}

// Rows above the row limit, one warp per piece of the row: each piece's
// minimum is folded into nf[v] (which k_sc_min set to f[v]) and, when it is
// below v's label, into the update addressed to that label; the minima over
// pieces are the row's minimum, so nf and upd end as with one pass per row.
template <bool CHECK>
__global__ void k_sc_min_pieces(uint64_t n, const uint64_t *__restrict__ rp,
                                const uint32_t *__restrict__ col, RowPieces rpc,
                                const uint32_t *__restrict__ f, uint32_t *nf, uint32_t *upd,
                                const uint32_t *__restrict__ act, int *err) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t ni = min((uint64_t)*rpc.count, rpc.cap);
  for (uint64_t h = warp; h < ni; h += nwarps) {
    uint32_t v;
    uint64_t b, e;
    row_piece(rpc, rp, h, v, b, e);
    if (act && !bit_of(act, v)) continue;  // warp-uniform: one row per piece
    bool bad = false;
    uint32_t best = piece_min_ilp<uint32_t>(col, b, e, lane, kNone, [&](uint32_t u) {
      if (CHECK && u >= n) {
        bad = true;
        return kNone;
      }
      return __ldg(f + u);
    });
    if (CHECK && bad) set_err(err, kErrBadId);
    best = __reduce_min_sync(0xffffffffu, best);
    if (lane == 0) {
      const uint32_t l = f[v];
      if (best < l) {
        atomicMin(nf + v, best);
        if (best < upd[l]) atomicMin(upd + l, best);  // entries only decrease
      }
    }
  }
}

// Heavy hitters (:210-223): labels held by more than n_part/h vertices.  The
// set is sticky across rounds as in the reference (heavy_hitters_ is never
// cleared).
__global__ void k_sc_count(uint64_t n, const uint32_t *__restrict__ nf, uint32_t *__restrict__ cnt) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + nf[v], 1u);
}
__global__ void k_sc_heavy(uint64_t n, const uint32_t *__restrict__ cnt, uint32_t thresh,
                           uint8_t *__restrict__ heavy) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    if (cnt[v] > thresh) heavy[v] = 1;
}

// The jump, the labels that changed (one bit per vertex in chg, whole words
// written by a warp) and their number (one atomic per block into *nchanged).
__global__ void k_sc_jump(uint64_t n, const uint32_t *__restrict__ f, uint32_t *__restrict__ nf,
                          const uint32_t *__restrict__ upd, const uint8_t *__restrict__ heavy,
                          uint32_t *__restrict__ chg, unsigned int *nchanged) {
  __shared__ unsigned int block_changed;
  if (threadIdx.x == 0) block_changed = 0;
  __syncthreads();
  const uint64_t span = (n + 31) / 32 * 32;  // warp-uniform trip count, 32-aligned lanes
  for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < span;
       u += (uint64_t)gridDim.x * blockDim.x) {
    bool changed = false;
    if (u < n) {
      const uint32_t t = nf[u];
      uint32_t r = t;
      if (!heavy || heavy[t]) {
        const uint32_t a = f[t];  // request l(l'(u)) answered by the owner of l'(u)
        r = a < r ? a : r;
      }
      const uint32_t up = upd[t];  // update messages addressed to target t
      r = up < r ? up : r;
      nf[u] = r;
      changed = r != f[u];
    }
    const unsigned b = __ballot_sync(0xffffffffu, changed);
    if ((threadIdx.x & 31) == 0) {
      chg[u >> 5] = b;
      if (b) atomicAdd(&block_changed, (unsigned)__popc(b));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && block_changed) atomicAdd(nchanged, block_changed);
}

// act |= the neighbours of every vertex whose bit is set in chg.  A row's ids
// are sorted, so runs of neighbours in one 32-vertex word are merged into
// one atomic; rows above the row limit go to k_mark_neighbours_pieces.
__global__ void k_mark_neighbours(uint64_t n, const uint64_t *__restrict__ rp,
                          const uint32_t *__restrict__ col, const uint32_t *__restrict__ chg,
                          uint32_t *act, uint64_t row_limit) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    if (!bit_of(chg, v)) continue;
    const uint64_t b = __ldg(rp + v), e = __ldg(rp + v + 1);
    if (e - b > row_limit) continue;
    uint32_t word = kNone, bits = 0;
    for (uint64_t k = b; k < e; ++k) {
      const uint32_t w = __ldg(col + k);
      if ((w >> 5) != word) {
        if (bits) atomicOr(act + word, bits);
        word = w >> 5;
        bits = 0;
      }
      bits |= 1u << (w & 31);
    }
    if (bits) atomicOr(act + word, bits);
  }
}
__global__ void k_mark_neighbours_pieces(const uint64_t *__restrict__ rp,
                                         const uint32_t *__restrict__ col, RowPieces rpc,
                                         const uint32_t *__restrict__ chg, uint32_t *act) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t ni = min((uint64_t)*rpc.count, rpc.cap);
  for (uint64_t h = warp; h < ni; h += nwarps) {
    uint32_t v;
    uint64_t b, e;
    row_piece(rpc, rp, h, v, b, e);
    if (!bit_of(chg, v)) continue;
    for (uint64_t k = b + lane; k < e; k += 32) {
      const uint32_t w = __ldg(col + k);
      atomicOr(act + (w >> 5), 1u << (w & 31));
    }
  }
}

// ---- composition / canonicalisation -----------------------------------------
__global__ void k_compose(uint64_t n, const uint32_t *__restrict__ cl,
                          const uint32_t *__restrict__ newid, const uint32_t *__restrict__ next,
                          const uint32_t *__restrict__ rep, uint32_t *__restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t c = cl[i];
    uint32_t id = newid[c];
    out[i] = id != kNone ? next[id] : (rep ? rep[c] : c);
  }
}

// mn[l] <- minimum v with lab[v] == l.  The test before the atomic reads
// through L1: mn only decreases, so a stale entry is never below the true one
// and a skip it allows is right; it keeps a giant component's entry from being
// one L2 line that every vertex reads.  Only a warp's smallest vertex of each
// label tests at all.
__global__ void k_canon_min(uint64_t n, uint32_t *mn, const uint32_t *__restrict__ lab) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t span = (n + 31) / 32 * 32;  // warp-uniform trip count
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < span; v += stride) {
    const bool in = v < n;
    const uint32_t l = in ? lab[v] : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, l);
    const bool first = (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1);
    if (in && first && (uint32_t)v < mn[l]) atomicMin(mn + l, (uint32_t)v);
  }
}
__global__ void k_canon_apply(uint64_t n, uint32_t *__restrict__ lab, const uint32_t *__restrict__ mn) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    lab[v] = mn[lab[v]];
}
__global__ void k_count_roots(uint64_t n, const uint32_t *__restrict__ lab,
                              unsigned long long *__restrict__ cnt) {
  unsigned long long c = 0;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    c += (lab[v] == (uint32_t)v);
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(__activemask(), c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, c);
}
// ---- component sizes (OutputComponents, static_graph.h:504-591) ------------
// cnt[l] = number of vertices labelled l.  A warp's lanes with the same label
// add once (labels come in runs: most vertices of a large component sit next
// to each other), so a giant component does not turn into one hot counter.
template <class T>
__global__ void k_comp_count(uint64_t n, const T *__restrict__ lab, uint32_t *__restrict__ cnt,
                             int *err) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n;
       base += stride) {
    const uint64_t v = base + lane;
    uint64_t l = v < n ? (uint64_t)lab[v] : ~0ull - lane;  // lanes past n match nothing
    if (v < n && l >= n) {
      set_err(err, kErrBadId);
      l = ~0ull - lane;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, l);
    if (l < n && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(cnt + l, (unsigned)__popc(peers));
  }
}
// hist[s] = number of labels held by s vertices (s >= 1), aggregated per warp
// the same way (most components are small, so a few sizes are hot).
__global__ void k_comp_hist(uint64_t n, const uint32_t *__restrict__ cnt, uint32_t *__restrict__ hist) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n;
       base += stride) {
    const uint64_t v = base + lane;
    const uint32_t c = v < n ? cnt[v] : 0u;
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    if (c && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(hist + c, (unsigned)__popc(peers));
  }
}

__global__ void k_gather(uint64_t n, const uint32_t *__restrict__ src, const uint32_t *__restrict__ idx,
                         uint32_t *__restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = src[idx[i]];
}
__global__ void k_iota(uint64_t n, uint32_t *__restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)i;
}

}  // namespace

int labels_propagate(const Csr &g, uint32_t *lab, int max_rounds, cudaStream_t s,
                     cudaMemPool_t pool, Counters &c, volatile int *host_flag, int *dev_flag) {
  if (g.n == 0) return 0;
  const uint32_t *col = static_cast<const uint32_t *>(g.col);
  unsigned grid = grid_for(g.n, kBlock, num_sms() * 32);
  const uint64_t cap = row_pieces_cap(g.m, kLabelRowLimit);
  const uint64_t words = (g.n + 31) / 32;
  DevBuf items(8 * cap, s, pool), cnt(4, s, pool), chga(4 * words, s, pool),
      chgb(4 * words, s, pool), actb(4 * words, s, pool);
  CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 4, s));
  const RowPieces rpc{items.as<uint2>(), cap, cnt.as<unsigned int>()};
  k_row_pieces<<<grid, kBlock, 0, s>>>(g.n, g.rp, kLabelRowLimit, rpc);
  CCG_LAUNCH_CHECK();
  uint32_t *chg = chga.as<uint32_t>(), *chg_prev = chgb.as<uint32_t>();
  unsigned int *nchanged = reinterpret_cast<unsigned int *>(dev_flag);
  int rounds = 0;
  bool sparse = false;  // visit only the neighbours of the labels lowered last round
  const uint64_t round_bytes = 8 * (g.n + 1) + g.m * 4 + g.m * 4 + 2 * g.n * 4;
  for (;;) {
    if (rounds >= max_rounds) return -1;
    CCG_CUDA(cudaMemsetAsync(dev_flag, 0, sizeof(int), s));
    CCG_CUDA(cudaMemsetAsync(chg, 0, 4 * words, s));
    if (sparse) {
      CCG_CUDA(cudaMemsetAsync(actb.p, 0, 4 * words, s));
      cudaEvent_t tp = c.tic(s);
      k_mark_neighbours<<<grid, kBlock, 0, s>>>(g.n, g.rp, col, chg_prev, actb.as<uint32_t>(),
                                                kLabelRowLimit);
      CCG_LAUNCH_CHECK();
      k_mark_neighbours_pieces<<<num_sms() * 8, kBlock, 0, s>>>(g.rp, col, rpc, chg_prev,
                                                        actb.as<uint32_t>());
      CCG_LAUNCH_CHECK();
      c.toc(s, "labels_push", tp, 0);
    }
    const uint32_t *act = sparse ? actb.as<uint32_t>() : nullptr;
    const bool check = g.err && rounds == 0;  // the caller's ids, not checked yet
    cudaEvent_t t0 = c.tic(s);
    if (check) {
      k_labels_round<true><<<grid, kBlock, 0, s>>>(g.n, g.rp, col, lab, act, chg, nchanged, g.err,
                                                    kLabelRowLimit);
      CCG_LAUNCH_CHECK();
      k_labels_round_pieces<true><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.rp, col, rpc, lab, act,
                                                                   chg, nchanged, g.err);
    } else {
      k_labels_round<false><<<grid, kBlock, 0, s>>>(g.n, g.rp, col, lab, act, chg, nchanged,
                                                    nullptr, kLabelRowLimit);
      CCG_LAUNCH_CHECK();
      k_labels_round_pieces<false><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.rp, col, rpc, lab, act,
                                                                    chg, nchanged, nullptr);
    }
    CCG_LAUNCH_CHECK();
    // algorithmic bytes of a round over every row (a round over the active
    // rows only is not counted)
    c.toc(s, "labels_round", t0, sparse ? 0 : round_bytes);
    CCG_CUDA(cudaMemcpyAsync((void *)host_flag, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (check)
      CCG_CUDA(cudaMemcpyAsync((void *)(host_flag + 1), g.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    if (check && host_flag[1] != 0) return kRoundsBadInput;
    ++rounds;
    c.add(2, round_bytes);
    const uint32_t changed = static_cast<uint32_t>(*host_flag);
    if (changed == 0) break;
    sparse = kLabelSparseDiv * changed <= g.n;
    uint32_t *t = chg;
    chg = chg_prev;
    chg_prev = t;
  }
  return rounds;
}

int shortcut_propagate(const Csr &g, uint32_t *lab, uint32_t hitters, int max_rounds,
                       cudaStream_t s, cudaMemPool_t pool, Counters &c, volatile int *host_flag,
                       int *dev_flag) {
  if (g.n == 0) return 0;
  const uint32_t *col = static_cast<const uint32_t *>(g.col);
  unsigned grid = grid_for(g.n, kBlock, num_sms() * 32);
  const uint64_t words = (g.n + 31) / 32;
  DevBuf nfb(4 * g.n, s, pool), updb(4 * g.n, s, pool), chgb(4 * words, s, pool),
      actb(4 * words, s, pool);
  const uint64_t cap = row_pieces_cap(g.m, kShortcutRowLimit);
  DevBuf items(8 * cap, s, pool), npieces(4, s, pool);
  const RowPieces rpc{items.as<uint2>(), cap, npieces.as<unsigned int>()};
  DevBuf cnt, heavy;
  if (hitters) {
    cnt.alloc(4 * g.n, s, pool);
    heavy.alloc(g.n, s, pool);
    CCG_CUDA(cudaMemsetAsync(heavy.p, 0, g.n, s));
  }
  CCG_CUDA(cudaMemsetAsync(npieces.p, 0, 4, s));
  k_row_pieces<<<grid, kBlock, 0, s>>>(g.n, g.rp, kShortcutRowLimit, rpc);
  CCG_LAUNCH_CHECK();
  uint32_t *f = lab, *nf = nfb.as<uint32_t>();
  const uint64_t min_bytes = 8 * (g.n + 1) + g.m * 4 + g.m * 4 + 2 * g.n * 4;
  int rounds = 0;
  bool sparse = false;  // visit only the rows next to a label changed last round
  for (;;) {
    if (rounds >= max_rounds) return -1;
    CCG_CUDA(cudaMemsetAsync(updb.p, 0xff, 4 * g.n, s));
    if (sparse) {
      CCG_CUDA(cudaMemsetAsync(actb.p, 0, 4 * words, s));
      cudaEvent_t tp = c.tic(s);
      k_mark_neighbours<<<grid, kBlock, 0, s>>>(g.n, g.rp, col, chgb.as<uint32_t>(),
                                                actb.as<uint32_t>(), kShortcutRowLimit);
      CCG_LAUNCH_CHECK();
      k_mark_neighbours_pieces<<<num_sms() * 8, kBlock, 0, s>>>(g.rp, col, rpc, chgb.as<uint32_t>(),
                                                        actb.as<uint32_t>());
      CCG_LAUNCH_CHECK();
      c.toc(s, "sc_push", tp, 0);
    }
    const uint32_t *act = sparse ? actb.as<uint32_t>() : nullptr;
    const bool check = g.err && rounds == 0;  // the caller's ids, not checked yet
    cudaEvent_t t0 = c.tic(s);
    if (check)
      k_sc_min<true><<<grid, kBlock, 0, s>>>(g.n, g.rp, col, f, nf, updb.as<uint32_t>(), act, g.err,
                                             kShortcutRowLimit);
    else
      k_sc_min<false><<<grid, kBlock, 0, s>>>(g.n, g.rp, col, f, nf, updb.as<uint32_t>(), act,
                                              nullptr, kShortcutRowLimit);
    CCG_LAUNCH_CHECK();
    // algorithmic bytes of a round over every row (a round over the active
    // rows only is not counted)
    c.toc(s, "sc_min", t0, sparse ? 0 : min_bytes);
    cudaEvent_t t0p = c.tic(s);
    if (check)
      k_sc_min_pieces<true><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.rp, col, rpc, f, nf,
                                                             updb.as<uint32_t>(), act, g.err);
    else
      k_sc_min_pieces<false><<<num_sms() * 8, kBlock, 0, s>>>(g.n, g.rp, col, rpc, f, nf,
                                                              updb.as<uint32_t>(), act, nullptr);
    CCG_LAUNCH_CHECK();
    c.toc(s, "sc_min_pieces", t0p, 0);
    cudaEvent_t t0j = c.tic(s);
    if (hitters) {
      CCG_CUDA(cudaMemsetAsync(cnt.p, 0, 4 * g.n, s));
      k_sc_count<<<grid, kBlock, 0, s>>>(g.n, nf, cnt.as<uint32_t>());
      CCG_LAUNCH_CHECK();
      k_sc_heavy<<<grid, kBlock, 0, s>>>(g.n, cnt.as<uint32_t>(), (uint32_t)(g.n / hitters),
                                         heavy.as<uint8_t>());
      CCG_LAUNCH_CHECK();
      c.add(2, 12 * g.n);
    }
    CCG_CUDA(cudaMemsetAsync(dev_flag, 0, sizeof(int), s));
    k_sc_jump<<<grid, kBlock, 0, s>>>(g.n, f, nf, updb.as<uint32_t>(),
                                      hitters ? heavy.as<uint8_t>() : nullptr, chgb.as<uint32_t>(),
                                      reinterpret_cast<unsigned int *>(dev_flag));
    CCG_LAUNCH_CHECK();
    c.toc(s, "sc_jump", t0j, 4 * g.n * 4 + 4 * g.n);
    CCG_CUDA(cudaMemcpyAsync((void *)host_flag, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (check)
      CCG_CUDA(cudaMemcpyAsync((void *)(host_flag + 1), g.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    if (check && host_flag[1] != 0) return kRoundsBadInput;
    ++rounds;
    // min sweep (offsets, ids, one label gather per edge, own r/w) + jump
    // (own label, two gathers, write)
    c.add(3, min_bytes + 4 * g.n * 4 + 4 * g.n);
    uint32_t *t = f;
    f = nf;
    nf = t;
    const uint32_t changed = static_cast<uint32_t>(*host_flag);  // labels lowered this round
    if (changed == 0) break;
    // when few labels changed, the next round pushes a mark to their
    // neighbours and visits only those rows (the first rounds lower nearly
    // every label and run over all rows)
    sparse = kShortcutSparseDiv * changed <= g.n;
  }
  if (f != lab) CCG_CUDA(cudaMemcpyAsync(lab, f, 4 * g.n, cudaMemcpyDeviceToDevice, s));
  return rounds;
}

void compose_labels(const uint32_t *cl, const uint32_t *newid, const uint32_t *next,
                    const uint32_t *rep, uint32_t *out, uint64_t n, cudaStream_t s, Counters &c) {
  if (n == 0) return;
  cudaEvent_t t0 = c.tic(s);
  k_compose<<<grid_for(n, kBlock, num_sms() * 32), kBlock, 0, s>>>(n, cl, newid, next, rep, out);
  CCG_LAUNCH_CHECK();
  c.toc(s, "compose", t0, 16 * n);
  c.add(1, 16 * n);
}

void canonicalize(uint32_t *lab, uint32_t *scratch, uint64_t n, cudaStream_t s, Counters &c) {
  if (n == 0) return;
  cudaEvent_t t0 = c.tic(s);
  CCG_CUDA(cudaMemsetAsync(scratch, 0xff, 4 * n, s));
  unsigned grid = grid_for(n, kBlock, num_sms() * 32);
  k_canon_min<<<grid, kBlock, 0, s>>>(n, scratch, lab);
  CCG_LAUNCH_CHECK();
  k_canon_apply<<<grid, kBlock, 0, s>>>(n, lab, scratch);
  CCG_LAUNCH_CHECK();
  c.toc(s, "canonicalize", t0, 4 * n * 4);
  c.add(2, 4 * n * 4);
}

void count_roots(const uint32_t *lab, uint64_t n, unsigned long long *d_count, cudaStream_t s,
                 Counters &c) {
  CCG_CUDA(cudaMemsetAsync(d_count, 0, 8, s));
  if (n == 0) return;
  k_count_roots<<<grid_for(n, kBlock, num_sms() * 8), kBlock, 0, s>>>(n, lab, d_count);
  CCG_LAUNCH_CHECK();
  c.add(1, 4 * n);
}

void component_size_hist(const void *lab, int id_bytes, uint64_t n, uint32_t *cnt, uint32_t *hist,
                         int *err, cudaStream_t s, Counters &c) {
  CCG_CUDA(cudaMemsetAsync(cnt, 0, 4 * n, s));
  CCG_CUDA(cudaMemsetAsync(hist, 0, 4 * (n + 1), s));
  if (n == 0) return;
  const unsigned grid = grid_for(n, kBlock, num_sms() * 16);
  if (id_bytes == 8)
    k_comp_count<uint64_t><<<grid, kBlock, 0, s>>>(n, static_cast<const uint64_t *>(lab), cnt, err);
  else
    k_comp_count<uint32_t><<<grid, kBlock, 0, s>>>(n, static_cast<const uint32_t *>(lab), cnt, err);
  CCG_LAUNCH_CHECK();
  k_comp_hist<<<grid, kBlock, 0, s>>>(n, cnt, hist);
  CCG_LAUNCH_CHECK();
  c.add(2, (uint64_t)id_bytes * n + 4 * n + 4 * n + 4 * n);
}

void gather_u32(const uint32_t *src, const uint32_t *idx, uint32_t *out, uint64_t n,
                cudaStream_t s, Counters &c) {
  if (n == 0) return;
  k_gather<<<grid_for(n, kBlock, num_sms() * 32), kBlock, 0, s>>>(n, src, idx, out);
  CCG_LAUNCH_CHECK();
  c.add(1, 12 * n);
}

void iota_u32(uint32_t *out, uint64_t n, cudaStream_t s, Counters &c) {
  if (n == 0) return;
  k_iota<<<grid_for(n, kBlock, num_sms() * 32), kBlock, 0, s>>>(n, out);
  CCG_LAUNCH_CHECK();
  c.add(1, 4 * n);
}

}  // namespace ccg

// api.cu - the C ABI of libccgpu and the solver orchestration.
//
// One call of cc_ctx_run() is one X(conf, rank, size).FindComponents(G,
// labels) of the reference (app/exp_contraction.cpp:104-105 and the other
// drivers), for one rank per GPU.  The five solver classes map to:
//
//   CC_EXP       ExponentialContraction::FindComponents
//                (exponential_contraction.h:59-319): partition-local CC,
//                component graph of the cut edges, exponential-shift
//                decomposition levels down to the sequential limit
//                (ComputeSequentialLimit :1287-1292), base case, labels
//                composed back up (UndoContraction) and applied to the input
//                (ApplyToLocalComponents :861-906).
//   CC_LOCAL     LocalContraction::FindComponents (local_contraction.h:52-91)
//   CC_SHORTCUTS ShortcutPropagation::FindComponents (shortcut_propagation.h:52-92)
//   CC_LABELS    Propagation::FindComponents (propagation.h:48-53)
//   CC_ALLREDUCE AllReduce<G>::FindComponents (all_reduce.h:46-76)
//
// Every path ends with canonical labels (minimum vertex id per component).
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>
#include <algorithm>

#include "../../include/cc_gpu_debug.h"
#include "ctx.h"

namespace ccg {
std::string &last_error() {
  static thread_local std::string s;
  return s;
}

void throw_on_kernel_error(cc_ctx *C, cudaStream_t s) {
  int e = 0;
  CCG_CUDA(cudaMemcpyAsync(&e, C->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CCG_CUDA(cudaStreamSynchronize(s));
  throw_on_error_word(e);
}

void throw_on_error_word(int e) {
  if (e == kErrBadOffsets) throw Error(CC_ERR_INVALID, "CSR offsets are not monotone or exceed m_dir");
  if (e == kErrBadId) throw Error(CC_ERR_INVALID, "CSR holds a vertex id >= n");
  if (e == kErrOverflow) throw Error(CC_ERR_INVALID, "CSR offsets disagree with m_dir");
  if (e) throw Error(CC_ERR_INVALID, "CSR check failed");
}

// Per-kernel CUDA-event times of c's records into st.kernels.
void collect_kernel_stats(Counters &c, cc_stats &st) {
  st.nkernels = 0;
  for (auto &r : c.recs) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    uint32_t k = 0;
    for (; k < st.nkernels; ++k)
      if (std::strncmp(st.kernels[k].name, r.name, sizeof(st.kernels[k].name)) == 0) break;
    if (k == st.nkernels) {
      if (st.nkernels >= CC_MAX_KSTATS) continue;
      std::memset(&st.kernels[k], 0, sizeof(st.kernels[k]));
      std::strncpy(st.kernels[k].name, r.name, sizeof(st.kernels[k].name) - 1);
      st.nkernels++;
    }
    st.kernels[k].launches += 1;
    st.kernels[k].ms += ms;
    st.kernels[k].bytes += r.bytes;
  }
  c.clear_recs();
}
}  // namespace ccg

namespace {

thread_local std::map<int, std::unique_ptr<cc_ctx>> g_default_ctx;
thread_local cc_stats g_last_stats{};

using ccg::Counters;
using ccg::Csr;
using ccg::DevBuf;
using ccg::Error;
using ccg::guard;
#define g_last_error (ccg::last_error())

void ctx_init(cc_ctx *c, int device, void *stream) {
  c->device = device;
  CCG_CUDA(cudaSetDevice(device));
  if (stream) {
    c->stream = static_cast<cudaStream_t>(stream);
  } else {
    CCG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  CCG_CUDA(cudaMemPoolCreate(&c->pool, &props));
  uint64_t thr = ~0ull;
  CCG_CUDA(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &thr));
  CCG_CUDA(cudaMalloc(&c->d_flag, sizeof(int)));
  CCG_CUDA(cudaMalloc(&c->d_err, sizeof(int)));
  CCG_CUDA(cudaMalloc(&c->d_geo, sizeof(uint64_t) * ccg::kGeoMax));
  CCG_CUDA(cudaHostAlloc(&c->h_flag, 2 * sizeof(int), cudaHostAllocDefault));  // flag, error word
  CCG_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  for (auto &e : c->ev) CCG_CUDA(cudaEventCreate(&e));
}

void ctx_free(cc_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  ccg::batch_cache_free(c->batch);
  c->batch = nullptr;
  c->plain_rp.release();
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->d_flag) cudaFree(c->d_flag);
  if (c->d_err) cudaFree(c->d_err);
  if (c->d_geo) cudaFree(c->d_geo);
  if (c->h_flag) cudaFreeHost(c->h_flag);
  if (c->pool) cudaMemPoolDestroy(c->pool);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  c->stager.reset();  // joins the host threads, frees the page-locked staging
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  c->ev_pool.clear();
}

void check_csr_args(const cc_csr *g) {
  if (!g) throw Error(CC_ERR_INVALID, "graph is NULL");
  if (g->id_bytes != 4 && g->id_bytes != 8) throw Error(CC_ERR_INVALID, "id_bytes must be 4 or 8");
  if (g->where != CC_HOST && g->where != CC_DEVICE) throw Error(CC_ERR_INVALID, "bad where");
  if (g->reserved != 0) throw Error(CC_ERR_INVALID, "reserved must be 0");
  if (g->num_parts == 0) throw Error(CC_ERR_INVALID, "num_parts must be >= 1");
  if (g->n >= 0xffffffffull)
    throw Error(CC_ERR_UNSUPPORTED, "n >= 2^32-1 vertices is not supported (uint32 labels inside)");
  if (g->n > 0 && !g->row_ptr) throw Error(CC_ERR_INVALID, "row_ptr is NULL");
  if (g->m_dir > 0 && !g->col) throw Error(CC_ERR_INVALID, "col is NULL");
  // the kernels load device offsets and ids as whole words (and ids in
  // 16-byte vectors from the first 16-byte boundary on); host arrays are
  // copied into fresh device buffers first
  if (g->where == CC_DEVICE) {
    if ((uintptr_t)g->row_ptr % 8 != 0) throw Error(CC_ERR_INVALID, "row_ptr is not 8-byte aligned");
    if ((uintptr_t)g->col % g->id_bytes != 0)
      throw Error(CC_ERR_INVALID, "col is not aligned to id_bytes");
  }
}

// Round cap of the iterative loops.  After r rounds every key (label) is at
// most the minimum over the r-hop neighbourhood, so each fixpoint is reached
// within n+1 rounds; hitting the cap means a fault, reported as
// CC_ERR_NO_CONVERGENCE.
// A context may lower it (cc_debug_set_round_cap) so that tests can reach the
// error path without a faulty kernel.
int round_cap(const cc_ctx *C, uint64_t n) {
  const uint64_t cap = std::min<uint64_t>(n + 2, 1u << 20);
  return (int)(C && C->round_cap ? std::min<uint64_t>(cap, C->round_cap) : cap);
}

// ---- the solvers -----------------------------------------------------------

struct Solver {
  cc_ctx *C;
  cudaStream_t s;
  cudaMemPool_t pool;
  Counters &c;
  const cc_config &cfg;
  uint64_t seed;
  cc_stats &st;
  uint64_t limit = 0;          // sequential limit (edges for CC_EXP, vertices for CC_LOCAL)
  ccg::UfTuning uf;            // hook-and-compress schedule (context tuning)
  const ccg::HostSource *hs = nullptr;  // streamed host input (tiled pass only)
  int max_levels = CC_MAX_LEVELS - 1;

  void check_err() { ccg::throw_on_kernel_error(C, s); }

  void note_level(uint32_t level, const Csr &G, int rounds) {
    if (level >= CC_MAX_LEVELS) return;
    st.level_vertices[level] = G.n;
    st.level_edges[level] = G.m;
    st.rounds[level] = rounds > 0 ? (uint32_t)rounds : 0u;
    if (level + 1 > st.levels) st.levels = level + 1;
    if (rounds > 0) st.rounds_total += (uint32_t)rounds;
    if (cfg.verbose)
      std::fprintf(stderr, "[cc] level %u: n=%llu m=%llu rounds=%d\n", level,
                   (unsigned long long)G.n, (unsigned long long)G.m, rounds);
  }

  // out[i] = vid[min index of i's component]  (RunSequentialCC ->
  // AllReduce::FindComponents, exponential_contraction.h:908-922)
  void base_case(const Csr &G, const uint32_t *vid, uint32_t *out) {
    DevBuf par(4 * G.n, s, pool);
    ccg::uf_components(G, par.as<uint32_t>(), nullptr, uf, s, pool, c);
    ccg::gather_u32(vid, par.as<uint32_t>(), out, G.n, s, c);
  }

  // RunContractionLP / RunContractionBFS recursion (exponential_contraction.h:
  // 364-389, 439-628): decompose, contract, recurse while m > limit.  Returns
  // true when no decomposition ran: out[i] is then vid of the smallest index
  // of i's component (base_case), which is the component's smallest original
  // id whenever vid increases with the index.
  bool exp_levels(const Csr &G, const uint32_t *vid, uint32_t level, uint32_t *out) {
    if (G.n == 0) return true;
    if (G.m <= limit || (int)level >= max_levels) {
      note_level(level, G, 0);
      base_case(G, vid, out);
      return true;
    }
    if (C->geo_beta != cfg.beta) {
      ccg::geo_table_upload(cfg.beta, C->d_geo, &C->geo_len, s);
      C->geo_beta = cfg.beta;
    }
    DevBuf cl(4 * G.n, s, pool);
    {
      DevBuf key(8 * G.n, s, pool);
      int rounds = ccg::ldd_decompose(G, vid, seed, level, C->d_geo, C->geo_len, cfg.bfs != 0,
                                      cl.as<uint32_t>(), key.as<uint64_t>(), round_cap(C, G.n), s, pool, c,
                                      C->h_flag, C->d_flag);
      if (rounds < 0) throw Error(CC_ERR_NO_CONVERGENCE, "decomposition did not converge");
      note_level(level, G, rounds);
    }
    ccg::Contracted H;
    ccg::contract_graph(G, cl.as<uint32_t>(), G.n, vid, nullptr, H, s, pool, c, nullptr);
    DevBuf sub(4 * (H.n ? H.n : 1), s, pool);
    Csr G2;
    G2.n = H.n;
    G2.m = H.m;
    G2.rp = H.rp.as<uint64_t>();
    G2.col = H.col.p;
    exp_levels(G2, H.vid.as<uint32_t>(), level + 1, sub.as<uint32_t>());
    ccg::compose_labels(cl.as<uint32_t>(), H.newid.as<uint32_t>(), sub.as<uint32_t>(), vid, out,
                        G.n, s, c);
    return false;
  }

  // LocalContraction::RunContraction recursion (local_contraction.h:157-300):
  // sweeps, contract, recurse while the vertex count exceeds the limit (an
  // absolute vertex count here, :119).
  void local_levels(const Csr &G, const uint32_t *vid, uint32_t level, uint32_t *out) {
    if (G.n == 0) return;
    if (G.n <= limit || G.m == 0 || (int)level >= max_levels) {
      note_level(level, G, 0);
      base_case(G, vid, out);
      return;
    }
    DevBuf cl(4 * G.n, s, pool);
    ccg::local_sweeps(G, vid, seed, level, cl.as<uint32_t>(), s, pool, c);
    if (G.err) check_err();  // the first sweep checked the caller's ids
    note_level(level, G, 2);
    ccg::Contracted H;
    ccg::contract_graph(G, cl.as<uint32_t>(), G.n, vid, nullptr, H, s, pool, c, nullptr);
    DevBuf sub(4 * (H.n ? H.n : 1), s, pool);
    Csr G2;
    G2.n = H.n;
    G2.m = H.m;
    G2.rp = H.rp.as<uint64_t>();
    G2.col = H.col.p;
    local_levels(G2, H.vid.as<uint32_t>(), level + 1, sub.as<uint32_t>());
    ccg::compose_labels(cl.as<uint32_t>(), H.newid.as<uint32_t>(), sub.as<uint32_t>(), vid, out,
                        G.n, s, c);
  }

  // Partition-local components and the component graph of the cut edges:
  // FindLocalComponents (exponential_contraction.h:391-411) followed by
  // CAGBuilder (cag_builder.h:69-73 local / :63-67 full CAG).  lab[v] = min id
  // of v's local component; G0 has one vertex per local component that owns a
  // cut edge, numbered by that id.
  void local_then_cut_graph(const Csr &g, uint32_t P, uint32_t *lab, ccg::Contracted &G0) {
    ccg::PartMap pm(g.n, P);
    ccg::uf_components(g, lab, &pm, uf, s, pool, c);
    check_err();  // the cut-edge pass reads the caller's ids again
    ccg::contract_graph(g, lab, g.n, nullptr, &pm, G0, s, pool, c, nullptr);
    note_level(0, g, 0);
  }

  // Caller graph as a trusted uint32 graph: checked, and 64-bit ids narrowed
  // into a copy (32-bit ids are used in place once the check has passed).
  // Caller graph as a uint32 graph for the propagation kernels.  64-bit ids
  // are checked and narrowed into a copy (h.err null: trusted).  32-bit ids
  // are used in place: the row offsets are checked here, the ids by the
  // first sweep that reads them (h.err stays set until then), which saves a
  // pass over the ids.
  Csr as_u32(const Csr &g, DevBuf &col32) {
    Csr h = g;
    h.idb = 4;
    if (g.idb != 4 || !g.err) {
      if (g.idb != 4) col32.alloc(4 * (g.m ? g.m : 1), s, pool);
      ccg::sanitize_ids(g, g.idb != 4 ? col32.as<uint32_t>() : nullptr, s, c);
      check_err();
      if (g.idb != 4) h.col = col32.p;
      h.err = nullptr;
    } else {
      ccg::check_offsets(g, s, c);
      check_err();
    }
    return h;
  }
  // Result of a round loop: a bad id found by its first round is reported
  // like any other input error.
  void rounds_ok(int r, const char *what) {
    if (r == ccg::kRoundsBadInput) check_err();
    if (r < 0) throw Error(CC_ERR_NO_CONVERGENCE, what);
  }

  void run(cc_algo algo, const Csr &g, uint32_t P, uint32_t *lab) {
    const uint64_t n = g.n;
    if (n == 0) return;
    switch (algo) {
      case CC_ALLREDUCE: {
        note_level(0, g, 0);
        ccg::uf_components(g, lab, nullptr, uf, s, pool, c, hs);
        break;
      }
      case CC_EXP: {
        // sequential_limit = fixed ? seq : (m/P)*seq  (:1287-1292)
        limit = cfg.fixed_seq ? (uint64_t)cfg.seq : (g.m / P) * (uint64_t)cfg.seq;
        if (P == 1) {
          // one rank: the local pass already is the whole solve, the component
          // graph has no edges (cag_builder.h:163-229)
          note_level(0, g, 0);
          ccg::uf_components(g, lab, nullptr, uf, s, pool, c, hs);
          break;
        }
        ccg::Contracted G0;
        local_then_cut_graph(g, P, lab, G0);
        if (G0.n) {
          DevBuf sub(4 * G0.n, s, pool);
          Csr G;
          G.n = G0.n;
          G.m = G0.m;
          G.rp = G0.rp.as<uint64_t>();
          G.col = G0.col.p;
          const bool direct = exp_levels(G, G0.vid.as<uint32_t>(), 1, sub.as<uint32_t>());
          ccg::compose_labels(lab, G0.newid.as<uint32_t>(), sub.as<uint32_t>(), nullptr, lab, n,
                              s, c);
          // Without a decomposition level the labels are canonical already:
          // G0 numbers the local components in increasing order of their
          // smallest ids (G0.vid increases), so the base case's smallest
          // index per component is the component's smallest vertex id.
          if (!direct) {
            DevBuf scratch(4 * n, s, pool);
            ccg::canonicalize(lab, scratch.as<uint32_t>(), n, s, c);
          }
        }
        break;
      }
      case CC_LOCAL: {
        limit = cfg.seq;  // absolute vertex count (local_contraction.h:119)
        if (cfg.contraction && P > 1) {
          ccg::Contracted G0;
          local_then_cut_graph(g, P, lab, G0);
          if (G0.n) {
            DevBuf sub(4 * G0.n, s, pool);
            Csr G;
            G.n = G0.n;
            G.m = G0.m;
            G.rp = G0.rp.as<uint64_t>();
            G.col = G0.col.p;
            local_levels(G, G0.vid.as<uint32_t>(), 1, sub.as<uint32_t>());
            ccg::compose_labels(lab, G0.newid.as<uint32_t>(), sub.as<uint32_t>(), nullptr, lab,
                                n, s, c);
          }
        } else {
          DevBuf col32, vid(4 * n, s, pool);
          Csr G = as_u32(g, col32);
          ccg::iota_u32(vid.as<uint32_t>(), n, s, c);
          local_levels(G, vid.as<uint32_t>(), 1, lab);
        }
        DevBuf scratch(4 * n, s, pool);
        ccg::canonicalize(lab, scratch.as<uint32_t>(), n, s, c);
        break;
      }
      case CC_SHORTCUTS: {
        if (cfg.contraction && P > 1) {
          ccg::Contracted G0;
          local_then_cut_graph(g, P, lab, G0);
          if (G0.n) {
            DevBuf f(4 * G0.n, s, pool), sub(4 * G0.n, s, pool);
            Csr G;
            G.n = G0.n;
            G.m = G0.m;
            G.rp = G0.rp.as<uint64_t>();
            G.col = G0.col.p;
            ccg::iota_u32(f.as<uint32_t>(), G0.n, s, c);
            int r = ccg::shortcut_propagate(G, f.as<uint32_t>(), cfg.number_of_hitters, round_cap(C, G.n),
                                            s, pool, c, C->h_flag, C->d_flag);
            if (r < 0) throw Error(CC_ERR_NO_CONVERGENCE, "shortcut propagation did not converge");
            note_level(1, G, r);
            ccg::gather_u32(G0.vid.as<uint32_t>(), f.as<uint32_t>(), sub.as<uint32_t>(), G0.n, s, c);
            ccg::compose_labels(lab, G0.newid.as<uint32_t>(), sub.as<uint32_t>(), nullptr, lab,
                                n, s, c);
          }
        } else {
          DevBuf col32;
          Csr G = as_u32(g, col32);
          ccg::iota_u32(lab, n, s, c);
          int r = ccg::shortcut_propagate(G, lab, cfg.number_of_hitters, round_cap(C, G.n), s, pool, c,
                                          C->h_flag, C->d_flag);
          rounds_ok(r, "shortcut propagation did not converge");
          note_level(0, G, r);
        }
        break;
      }
      case CC_LABELS: {
        DevBuf col32;
        Csr G = as_u32(g, col32);
        ccg::iota_u32(lab, n, s, c);
        uint64_t cap = C->round_cap ? std::min<uint64_t>(n + 2, C->round_cap) : n + 2;
        int r = ccg::labels_propagate(G, lab, (int)std::min<uint64_t>(cap, 0x7fffffff), s, pool, c,
                                      C->h_flag, C->d_flag);
        rounds_ok(r, "label propagation did not converge");
        note_level(0, G, r);
        break;
      }
      default:
        throw Error(CC_ERR_INVALID, "unknown algorithm");
    }
  }
};

// Adds one profiled solve to the context's running totals.
void accumulate_profile(cc_ctx *C, const cc_stats &st) {
  cc_stats &t = C->prof_total;
  for (uint32_t i = 0; i < st.nkernels; ++i) {
    uint32_t k = 0;
    for (; k < t.nkernels; ++k)
      if (std::strncmp(t.kernels[k].name, st.kernels[i].name, sizeof(t.kernels[k].name)) == 0) break;
    if (k == t.nkernels) {
      if (t.nkernels >= CC_MAX_KSTATS) continue;
      t.kernels[k] = st.kernels[i];
      t.nkernels++;
      continue;
    }
    t.kernels[k].launches += st.kernels[i].launches;
    t.kernels[k].ms += st.kernels[i].ms;
    t.kernels[k].bytes += st.kernels[i].bytes;
  }
  t.solve_ms += st.solve_ms;
  t.total_ms += st.total_ms;
  t.kernel_launches += st.kernel_launches;
  t.bytes_algorithmic += st.bytes_algorithmic;
  t.h2d_bytes += st.h2d_bytes;
  t.d2h_bytes += st.d2h_bytes;
  C->prof_solves++;
}

// Device address of a page-locked host range [p, p + bytes) that kernels on
// `device` may read: both ends registered with CUDA against that device and
// mapped at the same address (unified addressing), else false (pageable
// memory, memory of another device's context, or a range it cannot vouch for).
bool mapped_range(const void *p, size_t bytes, int device, const void **dev) {
  if (!p || bytes == 0) return false;
  const void *ends[2] = {p, static_cast<const char *>(p) + (bytes - 1)};
  for (const void *q : ends) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
      cudaGetLastError();  // an unknown pointer leaves a (non-sticky) error: clear it
      return false;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer != q || a.device != device) return false;
  }
  *dev = p;
  return true;
}

int ctx_run(cc_ctx *C, const cc_csr *g, cc_algo algo, const cc_config *cfg_in, uint64_t seed,
            void *labels_out, uint32_t labels_where) {
  return guard([&] {
    if (!C) throw Error(CC_ERR_INVALID, "context is NULL");
    check_csr_args(g);
    if (labels_where != CC_HOST && labels_where != CC_DEVICE)
      throw Error(CC_ERR_INVALID, "bad labels_where");
    if (g->n > 0 && !labels_out) throw Error(CC_ERR_INVALID, "labels_out is NULL");
    if ((int)algo < 0 || (int)algo > 4) throw Error(CC_ERR_INVALID, "unknown algorithm");
    cc_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else cc_config_default(&cfg);
    if (!(cfg.beta > 0.0) && algo == CC_EXP) throw Error(CC_ERR_INVALID, "beta must be > 0");
    CCG_CUDA(cudaSetDevice(C->device));
    cudaStream_t s = C->stream;
    cc_stats st;
    std::memset(&st, 0, sizeof(st));
    Counters c;
    c.prof = C->prof;
    c.pool = &C->ev_pool;
    const uint64_t n = g->n, m = g->m_dir;
    const int idb = (int)g->id_bytes;
    cudaEvent_t *ev = C->ev;  // the context's: no event creation per solve
    CCG_CUDA(cudaEventRecord(ev[0], s));
    DevBuf rp_d, col_d;
    Csr G;
    G.n = n;
    G.m = m;
    G.idb = idb;
    G.err = C->d_err;
    // Host input that suits the tiled pass (a sample of rows keeps most edges
    // inside their tile) is copied chunk by chunk while the tile kernel works
    // on the chunks already on the device.
    ccg::HostSource hsrc{g->row_ptr, g->col, C->copy_stream};
    bool streamed = false;
    if (g->where == CC_HOST && n > 0 && m > 0 &&
        (algo == CC_ALLREDUCE || (algo == CC_EXP && g->num_parts == 1))) {
      if (C->uf.mode == ccg::kUfTiled) {
        streamed = true;
      } else if (C->uf.mode == ccg::kUfAuto && n >= 4ull * C->uf.tile_vertices) {
        // the host sample (8192 scattered rows) is remembered like the
        // device one: a graph solved again from the same buffers skips it
        ccg::UfDecisionCache &dc = C->host_cache;
        if (!(dc.valid && dc.rp == g->row_ptr && dc.col == g->col && dc.n == n && dc.m == m &&
              dc.tile == C->uf.tile_vertices && dc.hub == C->uf.hub_degree)) {
          const ccg::HostShares hs = ccg::host_shares(g->row_ptr, g->col, idb, n, m,
                                                      C->uf.tile_vertices, C->uf.hub_degree);
          dc.rp = g->row_ptr;
          dc.col = g->col;
          dc.n = n;
          dc.m = m;
          dc.tile = C->uf.tile_vertices;
          dc.hub = C->uf.hub_degree;
          dc.tiles = hs.tiles;
          dc.link_tiles = hs.link_tiles;
          dc.few_hubs = hs.few_hubs;
          dc.valid = true;
        }
        // the tiled pass, or sampled linking whose link rounds stay in
        // their tiles: both run under the transfer
        streamed = dc.tiles || dc.link_tiles;
        hsrc.sampled = !dc.tiles;
      }
    }
    // Sampled linking reads each row's offsets and first entries, and whole
    // rows only outside the giant component: from page-locked host buffers
    // (mapped into the device's address space) the kernels read them in
    // place, so most of the ids never cross the host link.  (The tiled pass
    // reads every id: its input is copied, which measured faster than the
    // kernel's own reads across the link.)
    const void *rp_mapped = nullptr, *col_mapped = nullptr;
    if (streamed && hsrc.sampled && C->host_reads > 0 &&
        mapped_range(g->row_ptr, 8 * (n + 1), C->device, &rp_mapped) &&
        mapped_range(g->col, (size_t)idb * m, C->device, &col_mapped)) {
      hsrc.in_place = true;
      hsrc.offsets_copied = C->host_reads == 2;
    }
    if (streamed && (!hsrc.in_place || hsrc.offsets_copied)) {  // host threads encode the offsets as degree bytes
      if (!C->stager) C->stager.reset(new ccg::HostStager());
      hsrc.stager = C->stager.get();
    }
    if (hsrc.in_place && !hsrc.offsets_copied) {
      G.rp = static_cast<const uint64_t *>(rp_mapped);
      G.col = col_mapped;
    } else if (g->where == CC_HOST) {
      rp_d.alloc(8 * (n + 1), s, C->pool);
      if (!hsrc.in_place) col_d.alloc((size_t)idb * (m ? m : 1), s, C->pool);
      if (streamed) {
        // the copy stream may only write the buffers once they are allocated
        cudaEvent_t ev;
        CCG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        CCG_CUDA(cudaEventRecord(ev, s));
        CCG_CUDA(cudaStreamWaitEvent(C->copy_stream, ev, 0));
        cudaEventDestroy(ev);
      } else {
        if (n) CCG_CUDA(cudaMemcpyAsync(rp_d.p, g->row_ptr, 8 * (n + 1), cudaMemcpyHostToDevice, s));
        if (m) CCG_CUDA(cudaMemcpyAsync(col_d.p, g->col, (size_t)idb * m, cudaMemcpyHostToDevice, s));
      }
      st.h2d_bytes = n ? 8 * (n + 1) + (uint64_t)idb * m : 0;
      G.rp = rp_d.as<uint64_t>();
      G.col = hsrc.in_place ? col_mapped : col_d.p;
    } else {
      G.rp = g->row_ptr;
      G.col = g->col;
    }
    CCG_CUDA(cudaMemsetAsync(C->d_err, 0, sizeof(int), s));
    CCG_CUDA(cudaEventRecord(ev[1], s));
    // label array: the caller's buffer when it is a device uint32 array
    DevBuf lab_d;
    uint32_t *lab = nullptr;
    if (labels_where == CC_DEVICE && idb == 4) {
      lab = static_cast<uint32_t *>(labels_out);
    } else {
      lab_d.alloc(4 * (n ? n : 1), s, C->pool);
      lab = lab_d.as<uint32_t>();
    }
    // streamed uint32 host labels leave chunk by chunk under the final pass
    const bool labels_streamed = streamed && labels_where == CC_HOST && idb == 4 && n > 0;
    if (labels_streamed) hsrc.labels_out = labels_out;
    Solver S{C, s, C->pool, c, cfg, seed, st};
    S.uf = C->uf;
    S.uf.cache = &C->uf_cache;
    if (streamed) S.hs = &hsrc;
    S.run(algo, G, g->num_parts, lab);
    if (streamed) st.h2d_bytes = hsrc.h2d_bytes;  // offsets partly sent as degree bytes
    CCG_CUDA(cudaEventRecord(ev[2], s));
    DevBuf cnt(8, s, C->pool);
    if (C->prof_count) ccg::count_roots(lab, n, cnt.as<unsigned long long>(), s, c);
    if (labels_streamed) {
      st.d2h_bytes = 4 * n;  // copied by the final pass
    } else if (n) {
      if (labels_where == CC_DEVICE) {
        if (lab != labels_out) ccg::widen_labels(lab, labels_out, idb, n, s, c);
      } else {
        DevBuf wide;
        const void *src = lab;
        if (idb == 8) {
          wide.alloc(8 * n, s, C->pool);
          ccg::widen_labels(lab, wide.p, 8, n, s, c);
          src = wide.p;
        }
        CCG_CUDA(cudaMemcpyAsync(labels_out, src, (size_t)idb * n, cudaMemcpyDeviceToHost, s));
        st.d2h_bytes = (uint64_t)idb * n;
      }
    }
    CCG_CUDA(cudaEventRecord(ev[3], s));
    unsigned long long ncomp = 0;
    if (C->prof_count) CCG_CUDA(cudaMemcpyAsync(&ncomp, cnt.p, 8, cudaMemcpyDeviceToHost, s));
    // the error word rides along into pinned memory: one synchronisation ends the solve
    CCG_CUDA(cudaMemcpyAsync(C->h_flag + 1, C->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    ccg::throw_on_error_word(C->h_flag[1]);
    float t_solve = 0.f, t_total = 0.f;
    CCG_CUDA(cudaEventElapsedTime(&t_solve, ev[1], ev[2]));
    CCG_CUDA(cudaEventElapsedTime(&t_total, ev[0], ev[3]));
    st.solve_ms = t_solve;
    st.total_ms = t_total;
    st.bytes_algorithmic = c.bytes;
    st.kernel_launches = c.launches;
    st.num_components = ncomp;
    ccg::collect_kernel_stats(c, st);
    C->stats = st;
    if (C->prof) accumulate_profile(C, st);
  });
}

cc_ctx *default_ctx() {
  int dev = 0;
  CCG_CUDA(cudaGetDevice(&dev));
  auto &p = g_default_ctx[dev];
  if (!p) {
    std::unique_ptr<cc_ctx> c(new cc_ctx());
    try {
      ctx_init(c.get(), dev, nullptr);
    } catch (...) {
      ctx_free(c.get());
      throw;
    }
    p = std::move(c);
  }
  return p.get();
}

// ---- host-side CSR check ------------------------------------------------------
int validate_host(const cc_csr *g, int check_sym) {
  const uint64_t n = g->n, m = g->m_dir;
  if (n == 0) return m == 0 ? CC_OK : CC_ERR_INVALID;
  const uint64_t *rp = g->row_ptr;
  if (rp[0] != 0 || rp[n] != m) {
    g_last_error = "row_ptr[0] must be 0 and row_ptr[n] must equal m_dir";
    return CC_ERR_INVALID;
  }
  for (uint64_t v = 0; v < n; ++v)
    if (rp[v + 1] < rp[v]) {
      g_last_error = "row_ptr is not monotone";
      return CC_ERR_INVALID;
    }
  auto id = [&](uint64_t e) -> uint64_t {
    return g->id_bytes == 8 ? static_cast<const uint64_t *>(g->col)[e]
                            : static_cast<const uint32_t *>(g->col)[e];
  };
  for (uint64_t e = 0; e < m; ++e)
    if (id(e) >= n) {
      g_last_error = "vertex id >= n";
      return CC_ERR_INVALID;
    }
  if (check_sym) {
    std::vector<uint64_t> a, b;
    a.reserve(m);
    b.reserve(m);
    for (uint64_t v = 0; v < n; ++v)
      for (uint64_t e = rp[v]; e < rp[v + 1]; ++e) {
        uint64_t w = id(e);
        a.push_back((v << 32) | w);
        b.push_back((w << 32) | v);
      }
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b) {
      g_last_error = "CSR is not symmetric";
      return CC_ERR_INVALID;
    }
  }
  return CC_OK;
}

}  // namespace

namespace ccg {
cc_ctx *default_context() { return default_ctx(); }
}  // namespace ccg

// ============================== C ABI ========================================
extern "C" {

void cc_config_default(cc_config *cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->beta = 0.1;
  cfg->seq = 1;
  cfg->prop_iterations = 3;
  cfg->number_of_hitters = 0;
  cfg->degree_threshold = 16;
  cfg->degree_limit = 100;
  cfg->hd_sf = 0.5f;
}

int cc_ctx_create(cc_ctx **out, int device, void *stream) {
  if (!out) return CC_ERR_INVALID;
  *out = nullptr;
  std::unique_ptr<cc_ctx> c(new cc_ctx());
  int rc = guard([&] { ctx_init(c.get(), device, stream); });
  if (rc != CC_OK) {
    ctx_free(c.get());
    return rc;
  }
  *out = c.release();
  return CC_OK;
}

int cc_ctx_destroy(cc_ctx *ctx) {
  if (!ctx) return CC_ERR_INVALID;
  ctx_free(ctx);
  delete ctx;
  return CC_OK;
}

int cc_ctx_run(cc_ctx *ctx, const cc_csr *g, cc_algo algo, const cc_config *cfg, uint64_t seed,
               void *labels_out, uint32_t labels_where) {
  return ctx_run(ctx, g, algo, cfg, seed, labels_out, labels_where);
}

int cc_component_sizes(cc_ctx *ctx, const void *labels, uint32_t id_bytes, uint32_t where, uint64_t n,
                       uint64_t *pairs, uint64_t cap, uint64_t *npairs, uint64_t *num_components) {
  return guard([&] {
    if (id_bytes != 4 && id_bytes != 8) throw Error(CC_ERR_INVALID, "id_bytes must be 4 or 8");
    if (where != CC_HOST && where != CC_DEVICE) throw Error(CC_ERR_INVALID, "bad where");
    if (n > 0 && !labels) throw Error(CC_ERR_INVALID, "labels is NULL");
    if (cap > 0 && !pairs) throw Error(CC_ERR_INVALID, "pairs is NULL");
    if (!npairs) throw Error(CC_ERR_INVALID, "npairs is NULL");
    if (n >= 0xffffffffull) throw Error(CC_ERR_UNSUPPORTED, "n >= 2^32-1 labels is not supported");
    if (where == CC_DEVICE && (uintptr_t)labels % id_bytes != 0)
      throw Error(CC_ERR_INVALID, "labels are not aligned to id_bytes");
    cc_ctx *C = ctx ? ctx : default_ctx();
    CCG_CUDA(cudaSetDevice(C->device));
    cudaStream_t s = C->stream;
    Counters c;
    DevBuf lab_d;
    const void *lab = labels;
    if (where == CC_HOST && n) {
      lab_d.alloc((size_t)id_bytes * n, s, C->pool);
      CCG_CUDA(cudaMemcpyAsync(lab_d.p, labels, (size_t)id_bytes * n, cudaMemcpyHostToDevice, s));
      lab = lab_d.p;
    }
    // distinct sizes k_1 < ... < k_D of components that cover n vertices:
    // D (D + 1) / 2 <= n
    const uint64_t dmax = (uint64_t)std::sqrt(2.0 * (double)n) + 2;
    DevBuf cnt(4 * (n ? n : 1), s, C->pool), hist(4 * (n + 1), s, C->pool),
        out(16 * dmax, s, C->pool), dcount(4, s, C->pool);
    CCG_CUDA(cudaMemsetAsync(C->d_err, 0, sizeof(int), s));
    ccg::component_size_hist(lab, (int)id_bytes, n, cnt.as<uint32_t>(), hist.as<uint32_t>(),
                             C->d_err, s, c);
    ccg::compact_histogram(hist.as<uint32_t>(), n + 1, out.as<uint64_t>(), dmax,
                           dcount.as<uint32_t>(), s, C->pool, c);
    uint32_t d = 0;
    CCG_CUDA(cudaMemcpyAsync(&d, dcount.p, 4, cudaMemcpyDeviceToHost, s));
    ccg::throw_on_kernel_error(C, s);  // synchronises
    if (d > dmax) throw Error(CC_ERR_INVALID, "more distinct component sizes than n allows");
    std::vector<uint64_t> h(2 * (size_t)d);
    if (d) CCG_CUDA(cudaMemcpyAsync(h.data(), out.p, 16 * (size_t)d, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    uint64_t nontrivial = 0;  // the reference's NUM COMPONENTS leaves out isolated vertices
    for (uint32_t i = 0; i < d; ++i)
      if (h[2 * i] != 1) nontrivial += h[2 * i + 1];
    std::memcpy(pairs, h.data(), 16 * (size_t)std::min<uint64_t>(d, cap));
    *npairs = d;
    if (num_components) *num_components = nontrivial;
  });
}

int cc_ctx_stats(cc_ctx *ctx, cc_stats *out) {
  if (!ctx || !out) return CC_ERR_INVALID;
  *out = ctx->stats;
  return CC_OK;
}

uint64_t cc_ctx_arena_bytes(cc_ctx *ctx) {
  if (!ctx || !ctx->pool) return 0;
  uint64_t v = 0;
  cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrReservedMemCurrent, &v);
  return v;
}

int cc_ctx_set_profiling(cc_ctx *ctx, int on) {
  if (!ctx) return CC_ERR_INVALID;
  const bool kernels = (on & CC_PROF_KERNELS) != 0;
  if (kernels && !ctx->prof) {  // a new profiling window: the totals start from zero
    ctx->prof_total = cc_stats{};
    ctx->prof_solves = 0;
  }
  ctx->prof = kernels;
  ctx->prof_count = (on & CC_PROF_COMPONENTS) != 0;
  return CC_OK;
}

int cc_ctx_profile_totals(cc_ctx *ctx, cc_stats *out, uint64_t *solves) {
  if (!ctx || !out) return CC_ERR_INVALID;
  *out = ctx->prof_total;
  if (solves) *solves = ctx->prof_solves;
  return CC_OK;
}

void *cc_ctx_stream(cc_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int cc_ctx_set_tuning(cc_ctx *ctx, const cc_tuning *t) {
  if (!ctx || !t) return CC_ERR_INVALID;
  if (t->hook_mode > CC_HOOK_SAMPLED) return CC_ERR_INVALID;
  if ((t->tile_vertices && (t->tile_vertices < 32 || t->tile_vertices > 65536)) ||
      (t->tile_threads && (t->tile_threads % 32 || t->tile_threads > 1024)))
    return CC_ERR_INVALID;
  ccg::UfTuning u;
  u.mode = (int)t->hook_mode;
  if (t->tile_vertices) u.tile_vertices = t->tile_vertices;
  if (t->tile_threads) u.tile_threads = t->tile_threads;
  if (t->hub_degree) u.hub_degree = t->hub_degree;
  ctx->uf = u;
  return CC_OK;
}

int cc_ctx_set_host_reads(cc_ctx *ctx, int in_place) {
  if (!ctx || in_place < 0 || in_place > 2) return CC_ERR_INVALID;
  ctx->host_reads = in_place;
  return CC_OK;
}

int cc_ctx_get_tuning(cc_ctx *ctx, cc_tuning *t) {
  if (!ctx || !t) return CC_ERR_INVALID;
  t->hook_mode = (uint32_t)ctx->uf.mode;
  t->tile_vertices = ctx->uf.tile_vertices;
  t->tile_threads = ctx->uf.tile_threads;
  t->hub_degree = ctx->uf.hub_degree;
  return CC_OK;
}

int cc_gpu_run(const cc_csr *g, cc_algo algo, const cc_config *cfg, uint64_t seed,
               void *labels_out) {
  cc_ctx *C = nullptr;
  int rc = guard([&] { C = default_ctx(); });
  if (rc != CC_OK) return rc;
  rc = ctx_run(C, g, algo, cfg, seed, labels_out, g ? g->where : CC_HOST);
  g_last_stats = C->stats;
  return rc;
}

int cc_gpu_stats(cc_stats *out) {
  if (!out) return CC_ERR_INVALID;
  *out = g_last_stats;
  return CC_OK;
}

const char *cc_gpu_strerror(int status) {
  switch (status) {
    case CC_OK: return "ok";
    case CC_ERR_INVALID: return g_last_error.empty() ? "invalid argument" : g_last_error.c_str();
    case CC_ERR_OOM: return "out of memory";
    case CC_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
    case CC_ERR_NO_CONVERGENCE: return "iteration cap reached without convergence";
    case CC_ERR_TIMEOUT: return "bounded device wait gave up";
    case CC_ERR_UNSUPPORTED: return g_last_error.empty() ? "unsupported" : g_last_error.c_str();
    case CC_ERR_BUSY: return "busy";
    default: return "unknown status";
  }
}

int cc_csr_validate(const cc_csr *g, int check_sym) {
  int rc = guard([&] { check_csr_args(g); });
  if (rc != CC_OK) return rc;
  if (g->where == CC_HOST) return validate_host(g, check_sym);
  // device graph: copy to the host and check there
  std::vector<uint64_t> rp(g->n + 1);
  std::vector<uint8_t> col((size_t)g->id_bytes * g->m_dir);
  rc = guard([&] {
    if (g->n) CCG_CUDA(cudaMemcpy(rp.data(), g->row_ptr, 8 * (g->n + 1), cudaMemcpyDeviceToHost));
    if (g->m_dir) CCG_CUDA(cudaMemcpy(col.data(), g->col, col.size(), cudaMemcpyDeviceToHost));
  });
  if (rc != CC_OK) return rc;
  cc_csr h = *g;
  h.row_ptr = rp.data();
  h.col = col.data();
  h.where = CC_HOST;
  return validate_host(&h, check_sym);
}

// ---- test hooks (cc_gpu_debug.h) ---------------------------------------------

int cc_debug_geo_table(double beta, uint64_t *out, int cap) {
  std::vector<uint64_t> t;
  int len = ccg::geo_table_build(beta, t);
  if (out)
    for (int i = 0; i < len && i < cap; ++i) out[i] = t[i];
  return len;
}

uint64_t cc_debug_hash3(uint64_t seed, uint64_t a, uint64_t b) { return ccg::hash3(seed, a, b); }

static Csr dev_u32_graph(const cc_csr *g) {
  check_csr_args(g);
  if (g->where != CC_DEVICE || g->id_bytes != 4)
    throw Error(CC_ERR_INVALID, "debug hooks take device graphs with uint32 ids");
  Csr G;
  G.n = g->n;
  G.m = g->m_dir;
  G.rp = g->row_ptr;
  G.col = g->col;
  G.idb = 4;
  return G;
}

int cc_debug_ldd(const cc_csr *g, const uint32_t *vid, uint64_t seed, uint32_t level, double beta,
                 int gated, uint32_t *cluster_out, uint32_t *rounds_out) {
  return guard([&] {
    Csr G = dev_u32_graph(g);
    cc_ctx *C = default_ctx();
    cudaStream_t s = C->stream;
    if (C->geo_beta != beta) {
      ccg::geo_table_upload(beta, C->d_geo, &C->geo_len, s);
      C->geo_beta = beta;
    }
    Counters c;
    DevBuf key(8 * (G.n ? G.n : 1), s, C->pool);
    int r = ccg::ldd_decompose(G, vid, seed, level, C->d_geo, C->geo_len, gated != 0, cluster_out,
                               key.as<uint64_t>(), round_cap(C, G.n), s, C->pool, c, C->h_flag, C->d_flag);
    CCG_CUDA(cudaStreamSynchronize(s));
    if (r < 0) throw Error(CC_ERR_NO_CONVERGENCE, "decomposition did not converge");
    if (rounds_out) *rounds_out = (uint32_t)r;
  });
}

int cc_debug_local_sweeps(const cc_csr *g, const uint32_t *vid, uint64_t seed, uint32_t level,
                          uint32_t *cluster_out) {
  return guard([&] {
    Csr G = dev_u32_graph(g);
    cc_ctx *C = default_ctx();
    cudaStream_t s = C->stream;
    Counters c;
    ccg::local_sweeps(G, vid, seed, level, cluster_out, s, C->pool, c);
    CCG_CUDA(cudaStreamSynchronize(s));
  });
}

int cc_debug_contract(const cc_csr *g, const uint32_t *cl, uint64_t ncl,
                      const uint32_t *vid_of_cluster, uint32_t cut_parts, uint64_t *rp_out,
                      uint32_t *col_out, uint32_t *vid_out, uint32_t *newid_out, uint64_t *n_out,
                      uint64_t *m_out) {
  return guard([&] {
    check_csr_args(g);
    if (g->where != CC_DEVICE) throw Error(CC_ERR_INVALID, "debug hooks take device graphs");
    Csr G;
    G.n = g->n;
    G.m = g->m_dir;
    G.rp = g->row_ptr;
    G.col = g->col;
    G.idb = (int)g->id_bytes;
    cc_ctx *C = default_ctx();
    cudaStream_t s = C->stream;
    Counters c;
    ccg::Contracted H;
    ccg::PartMap pm(g->n, cut_parts ? cut_parts : 1);
    ccg::contract_graph(G, cl, ncl, vid_of_cluster, cut_parts ? &pm : nullptr, H, s, C->pool, c,
                        nullptr);
    CCG_CUDA(cudaMemcpyAsync(rp_out, H.rp.p, 8 * (H.n + 1), cudaMemcpyDeviceToDevice, s));
    if (H.m) CCG_CUDA(cudaMemcpyAsync(col_out, H.col.p, 4 * H.m, cudaMemcpyDeviceToDevice, s));
    if (H.n) CCG_CUDA(cudaMemcpyAsync(vid_out, H.vid.p, 4 * H.n, cudaMemcpyDeviceToDevice, s));
    if (ncl) CCG_CUDA(cudaMemcpyAsync(newid_out, H.newid.p, 4 * ncl, cudaMemcpyDeviceToDevice, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    *n_out = H.n;
    *m_out = H.m;
  });
}

int cc_debug_local_components(const cc_csr *g, uint32_t *labels_out) {
  return guard([&] {
    check_csr_args(g);
    if (g->where != CC_DEVICE) throw Error(CC_ERR_INVALID, "debug hooks take device graphs");
    Csr G;
    G.n = g->n;
    G.m = g->m_dir;
    G.rp = g->row_ptr;
    G.col = g->col;
    G.idb = (int)g->id_bytes;
    cc_ctx *C = default_ctx();
    cudaStream_t s = C->stream;
    G.err = C->d_err;
    CCG_CUDA(cudaMemsetAsync(C->d_err, 0, sizeof(int), s));
    Counters c;
    ccg::PartMap pm(g->n, g->num_parts);
    ccg::uf_components(G, labels_out, g->num_parts > 1 ? &pm : nullptr, C->uf, s, C->pool, c);
    int e = 0;
    CCG_CUDA(cudaMemcpyAsync(&e, C->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    if (e) throw Error(CC_ERR_INVALID, "CSR check failed");
  });
}

int cc_debug_radix_sort(uint64_t *keys, uint64_t n, int bits) {
  return guard([&] {
    cc_ctx *C = default_ctx();
    cudaStream_t s = C->stream;
    Counters c;
    DevBuf tmp(8 * (n ? n : 1), s, C->pool);
    uint64_t *r = ccg::radix_sort_u64(keys, tmp.as<uint64_t>(), n, bits, s, C->pool, c);
    if (r != keys) CCG_CUDA(cudaMemcpyAsync(keys, r, 8 * n, cudaMemcpyDeviceToDevice, s));
    CCG_CUDA(cudaStreamSynchronize(s));
  });
}

int cc_debug_set_round_cap(cc_ctx *ctx, uint32_t cap) {
  if (!ctx) return CC_ERR_INVALID;
  ctx->round_cap = cap;
  return CC_OK;
}

int cc_debug_shortcut(const cc_csr *g, uint32_t *labels_inout, uint32_t hitters,
                      uint32_t *rounds_out) {
  return guard([&] {
    Csr G = dev_u32_graph(g);
    cc_ctx *C = default_ctx();
    cudaStream_t s = C->stream;
    Counters c;
    int r = ccg::shortcut_propagate(G, labels_inout, hitters, round_cap(C, G.n), s, C->pool, c, C->h_flag,
                                    C->d_flag);
    CCG_CUDA(cudaStreamSynchronize(s));
    if (r < 0) throw Error(CC_ERR_NO_CONVERGENCE, "shortcut propagation did not converge");
    if (rounds_out) *rounds_out = (uint32_t)r;
  });
}

}  // extern "C"

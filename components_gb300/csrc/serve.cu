// serve.cu - continuous-batching CC server (include/cc_serve.h).
//
// No counterpart in the reference.  One worker thread per server:
//   admission  requests wait on the host in arrival order until their device
//              bytes fit the HBM budget; then their CSR is copied to the device
//              on the copy stream (an event marks the copy)
//   batching   whenever one of the compute streams has finished its previous
//              batch, every staged request (up to max_batch_graphs) is
//              coalesced into one launch on it: graphs up to smem_max_n
//              vertices and 32768 entries are solved one CTA each (union-find
//              in shared memory, CTAs pull graphs from a queue), larger ones by
//              the grid-wide hook-and-compress; the stream first waits on the
//              copy events
//   completion a host callback after the batch marks its requests done
//   collect    the client copies the labels back, which frees the request's
//              device memory and budget
// Copies of new requests overlap the batches already running, and several
// compute streams (four by default) let batches overlap on the device, so a
// small request does not wait for a stream that is busy with large graphs.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cc_serve.h"
#include "ctx.h"

namespace ccg {
struct Server;
namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct GraphDesc {
  const uint64_t *rp;  // local offsets (rp[0] == 0)
  const void *col;     // local ids
  uint32_t *labels;    // n labels, then the request's error word
  uint64_t m;
  uint32_t n;
  uint32_t idb;
};

// One CTA per small graph of the batch; persistent CTAs pull descriptors.
__global__ void k_serve_smem(const GraphDesc *__restrict__ descs, uint32_t count,
                             unsigned int *__restrict__ queue) {
  extern __shared__ uint32_t sp[];
  __shared__ uint32_t item;
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(queue, 1u);
    __syncthreads();
    const uint32_t it = item;
    __syncthreads();
    if (it >= count) return;
    const GraphDesc d = descs[it];
    int *err = reinterpret_cast<int *>(d.labels + d.n);
    volatile uint32_t *p = sp;
    for (uint32_t v = threadIdx.x; v < d.n; v += blockDim.x) p[v] = v;
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < d.n; v += blockDim.x) {
      uint64_t b = d.rp[v], e = d.rp[v + 1];
      if (e < b || e > d.m) {
        set_err(err, kErrBadOffsets);
        continue;
      }
      for (uint64_t k = b; k < e; ++k) {
        uint64_t u = d.idb == 8 ? static_cast<const uint64_t *>(d.col)[k]
                                : static_cast<const uint32_t *>(d.col)[k];
        if (u >= d.n) {
          set_err(err, kErrBadId);
          continue;
        }
        if (u < v) smem_union<false>(p, v, (uint32_t)u);
      }
    }
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < d.n; v += blockDim.x) {
      uint32_t r = v, nx;
      while ((nx = p[r]) != r) r = nx;
      d.labels[v] = r;
    }
    __syncthreads();
  }
}

enum ReqState { kWaiting = 0, kStaged = 1, kLaunched = 2, kDone = 3 };
constexpr uint64_t kSmemMaxEntries = 32768;
constexpr double kAdmitSlice = 300e-6;  // seconds of staging before a free stream gets work

struct Req {
  uint64_t id = 0;
  cc_csr g{};
  uint64_t need = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  DevBuf rp, col, lab;  // lab: n labels + error word
  cudaEvent_t copied = nullptr;
  std::atomic<int> state{kWaiting};
  uint32_t batch_id = 0, batch_size = 0;
  bool failed = false;    // could not be staged or launched (collect reports fail_status)
  int fail_status = CC_ERR_CUDA;
  int inject = 0;         // test hook: fail on purpose at staging (1) or launch (2)
  bool enqueued = false;  // its completion callback is queued on a stream
  UfTuning tu;  // large graph: hook schedule decided on the host
};

struct Batch {
  std::vector<Req *> reqs;
  Server *srv = nullptr;
  int stream = 0;
};

}  // namespace

struct Server {
  int device = 0;
  cc_serve_config cfg{};
  cudaMemPool_t pool = nullptr;
  cudaStream_t copy_stream = nullptr, collect_stream = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<std::atomic<int>> busy;  // batches in flight per compute stream
  std::vector<DevBuf> desc_dev, queue_dev;
  std::vector<GraphDesc *> desc_host;  // pinned
  std::mutex mu;
  std::condition_variable cv_worker, cv_done;
  std::deque<Req *> waiting, staged;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  uint64_t next_id = 1, used = 0, peak = 0, batches = 0, submitted = 0, completed = 0,
           collected = 0;
  bool stop = false;
  std::atomic<int> inject_next{0};  // test hook (cc_serve_debug_fail_next)
  std::thread worker;
  std::atomic<int> inflight{0};

  explicit Server(size_t ns) : busy(ns) {}

  static void CUDART_CB on_batch_done(void *arg) {
    std::unique_ptr<Batch> b(static_cast<Batch *>(arg));
    Server *s = b->srv;
    double t = now_s();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (Req *r : b->reqs) {
        r->t_done = t;
        r->state = kDone;
      }
      s->completed += b->reqs.size();
    }
    s->busy[b->stream]--;
    s->inflight--;
    s->cv_done.notify_all();
    s->cv_worker.notify_all();
  }

  // Solved by one CTA in shared memory: at most smem_max_n vertices and
  // kSmemMaxEntries entries.  One CTA walks a graph's entries at the latency of
  // its own loads (a lone graph of 200,000 entries took 2 ms that way); the
  // grid-wide path solves it in a fraction of that.
  bool small(const cc_csr &g) const { return g.n <= cfg.smem_max_n && g.m_dir <= kSmemMaxEntries; }

  uint64_t bytes_needed(const cc_csr &g) const {
    uint64_t b = 8 * (g.n + 1) + (uint64_t)g.id_bytes * g.m_dir + 4 * (g.n + 1) + 3 * 256;
    if (!small(g))  // hook scratch: cut list and hub pieces
      b += 8 * (g.m_dir + 1) + 8 * (g.m_dir / 33 + g.m_dir / 2048 + 2) + 8192;
    return b;
  }

  // Hook schedule of a large graph, decided on the host CSR without a device
  // round trip, by the rule of the auto schedule: the tiled pass when a row
  // sample suits it, the global hook when the graph is L2-resident with few
  // hub rows, else sampled linking (with tiled link rounds when they stay in
  // their tile).
  static UfTuning schedule(const cc_csr &g) {
    UfTuning tu;
    // 512 rows: the shares are compared with 50 %, 25 % and 10 % (a 512-row
    // sample of rows with a few entries each is within about 2 % of them), and
    // the sample runs on the submitting thread over a CSR that is cold in the
    // host caches: 2048 rows cost about 0.4 ms a request there
    const HostShares sh = host_shares(g.row_ptr, g.col, (int)g.id_bytes, g.n, g.m_dir,
                                      tu.tile_vertices, tu.hub_degree, 512);
    const uint64_t ws = 8 * (g.n + 1) + g.m_dir * (uint64_t)g.id_bytes + 4 * g.n;
    if (g.n >= 4ull * tu.tile_vertices && sh.tiles) tu.mode = kUfTiled;
    else if (ws <= (96ull << 20) && sh.few_hubs) tu.mode = kUfGlobal;
    else tu.mode = kUfSampled;
    tu.link_tiles = g.n >= 4ull * tu.tile_vertices && sh.link_tiles ? 1 : 0;
    return tu;
  }

  void stage(Req *r) {  // worker thread, no lock held
    const cc_csr &g = r->g;
    if (r->inject == 1) throw Error(CC_ERR_OOM, "injected staging failure (test hook)");
    r->rp.alloc(8 * (g.n + 1), copy_stream, pool);
    r->col.alloc((size_t)g.id_bytes * (g.m_dir ? g.m_dir : 1), copy_stream, pool);
    r->lab.alloc(4 * (g.n + 1), copy_stream, pool);
    CCG_CUDA(cudaMemcpyAsync(r->rp.p, g.row_ptr, 8 * (g.n + 1), cudaMemcpyHostToDevice, copy_stream));
    if (g.m_dir)
      CCG_CUDA(cudaMemcpyAsync(r->col.p, g.col, (size_t)g.id_bytes * g.m_dir,
                               cudaMemcpyHostToDevice, copy_stream));
    CCG_CUDA(cudaMemsetAsync(r->lab.as<uint32_t>() + g.n, 0, 4, copy_stream));
    CCG_CUDA(cudaEventCreateWithFlags(&r->copied, cudaEventDisableTiming));
    CCG_CUDA(cudaEventRecord(r->copied, copy_stream));
  }

  // A request that could not be launched: done, reported as failed by collect.
  void fail(Req *r) {
    {
      std::lock_guard<std::mutex> lk(mu);
      r->failed = true;
      r->batch_id = 0;
      r->t_done = now_s();
      r->state = kDone;
    }
    cv_done.notify_all();
  }

  // Completion of `reqs` once stream s reaches this point (a host callback).
  void enqueue_done(std::vector<Req *> reqs, int si, cudaStream_t s) {
    Batch *b = new Batch{std::move(reqs), this, si};
    busy[si]++;
    inflight++;
    for (Req *r : b->reqs) r->enqueued = true;
    if (cudaLaunchHostFunc(s, on_batch_done, b) != cudaSuccess) {
      busy[si]--;
      inflight--;
      for (Req *r : b->reqs) fail(r);
      delete b;
    }
  }

  // One launch sequence on compute stream si: the small graphs (one CTA each in
  // shared memory) complete together as soon as their kernel ends; every large
  // graph completes on its own after its hook pass, so small requests never
  // wait behind a large one in the same launch.  Never throws: a request whose
  // part cannot be launched is failed alone.
  void launch(std::vector<Req *> &batch, int si) {  // worker thread, no lock held
    cudaStream_t s = streams[si];
    std::stable_partition(batch.begin(), batch.end(),
                          [&](Req *r) { return small(r->g); });
    {
      std::lock_guard<std::mutex> lk(mu);
      const uint32_t bid = (uint32_t)++batches;
      for (Req *r : batch) {
        r->batch_id = bid;
        r->batch_size = (uint32_t)batch.size();
        r->state = kLaunched;
      }
    }
    GraphDesc *hd = desc_host[si];
    uint32_t nsmall = 0;
    for (Req *r : batch)
      if (small(r->g)) ++nsmall;
    Counters c;
    if (nsmall) {
      std::vector<Req *> smalls(batch.begin(), batch.begin() + nsmall);
      try {
        for (uint32_t i = 0; i < nsmall; ++i) {
          Req *r = batch[i];
          CCG_CUDA(cudaStreamWaitEvent(s, r->copied, 0));
          hd[i] = GraphDesc{r->rp.as<uint64_t>(), r->col.p, r->lab.as<uint32_t>(), r->g.m_dir,
                            (uint32_t)r->g.n, r->g.id_bytes};
        }
        CCG_CUDA(cudaMemcpyAsync(desc_dev[si].p, hd, sizeof(GraphDesc) * nsmall,
                                 cudaMemcpyHostToDevice, s));
        CCG_CUDA(cudaMemsetAsync(queue_dev[si].p, 0, 4, s));
        const size_t smem = 4ull * cfg.smem_max_n;
        if (smem > 48 * 1024)
          CCG_CUDA(cudaFuncSetAttribute(k_serve_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
        int per_sm = 1;
        CCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_serve_smem, 256, smem));
        unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)std::max(per_sm, 1) * num_sms(), nsmall);
        k_serve_smem<<<grid, 256, smem, s>>>(desc_dev[si].as<GraphDesc>(), nsmall,
                                             queue_dev[si].as<unsigned int>());
        CCG_LAUNCH_CHECK();
        enqueue_done(std::move(smalls), si, s);
      } catch (...) {
        for (Req *r : smalls) fail(r);
      }
    }
    for (size_t i = nsmall; i < batch.size(); ++i) {
      Req *r = batch[i];
      try {
        if (r->inject == 2) throw Error(CC_ERR_CUDA, "injected launch failure (test hook)");
        CCG_CUDA(cudaStreamWaitEvent(s, r->copied, 0));
        Csr G;
        G.n = r->g.n;
        G.m = r->g.m_dir;
        G.rp = r->rp.as<uint64_t>();
        G.col = r->col.p;
        G.idb = (int)r->g.id_bytes;
        G.err = reinterpret_cast<int *>(r->lab.as<uint32_t>() + r->g.n);
        // schedule decided on the host: no device round trip in the loop
        uf_components(G, r->lab.as<uint32_t>(), nullptr, r->tu, s, pool, c);
      } catch (...) {
        fail(r);
        continue;
      }
      enqueue_done({r}, si, s);
    }
  }

  void loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_worker.wait_for(lk, std::chrono::microseconds(500), [&] {
        bool admit = !waiting.empty() && used + waiting.front()->need <= cfg.hbm_budget_bytes;
        bool free_stream = false;
        for (auto &b : busy) free_stream |= b.load() == 0;
        return stop || admit || (!staged.empty() && free_stream);
      });
      if (stop && waiting.empty() && staged.empty()) break;
      // admission, in arrival order, while the budget allows.  Staging is host
      // work (a large request's copy and schedule take up to 1.6 ms), so during
      // a burst the worker stops admitting after kAdmitSlice seconds whenever a
      // compute stream is free, launches what is staged, and comes back: the
      // first requests of a burst do not wait for the last ones to be staged.
      const double t_admit0 = now_s();
      while (!waiting.empty() && used + waiting.front()->need <= cfg.hbm_budget_bytes) {
        if (!staged.empty() && now_s() - t_admit0 > kAdmitSlice) {
          bool free_stream = false;
          for (auto &b : busy) free_stream |= b.load() == 0;
          if (free_stream) break;
        }
        Req *r = waiting.front();
        waiting.pop_front();
        used += r->need;
        peak = std::max(peak, used);
        r->t_admit = now_s();
        lk.unlock();
        int st = CC_OK;
        try {
          stage(r);
        } catch (const Error &e) {
          st = e.status;
        } catch (...) {
          st = CC_ERR_CUDA;
        }
        if (st != CC_OK) {
          // the copy stream is left to finish what was enqueued; collect
          // reports the status and retires the request (its buffers and its
          // share of the budget)
          lk.lock();
          r->failed = true;
          r->fail_status = st;
          r->t_done = now_s();
          r->state = kDone;
          cv_done.notify_all();
          continue;
        }
        lk.lock();
        r->state = kStaged;
        staged.push_back(r);
      }
      // batching window: let more requests arrive unless the batch is full
      if (!staged.empty() && cfg.batch_window_us && staged.size() < cfg.max_batch_graphs &&
          (now_s() - staged.front()->t_admit) * 1e6 < cfg.batch_window_us && !stop) {
        cv_worker.wait_for(lk, std::chrono::microseconds(50));
        continue;
      }
      // batching: every free compute stream takes the staged requests
      for (size_t si = 0; si < streams.size() && !staged.empty(); ++si) {
        if (busy[si].load() > 0) continue;
        std::vector<Req *> batch;
        while (!staged.empty() && batch.size() < cfg.max_batch_graphs) {
          batch.push_back(staged.front());
          staged.pop_front();
        }
        lk.unlock();
        try {
          launch(batch, (int)si);
        } catch (...) {
          // launch fails requests itself; this only catches a host allocation
          // failure, after which no completion may be pending for the rest
          for (Req *r : batch)
            if (!r->enqueued && r->state.load() != kDone) fail(r);
        }
        lk.lock();
      }
    }
  }
};

}  // namespace ccg

struct cc_server {
  std::unique_ptr<ccg::Server> s;
};

extern "C" {

void cc_serve_config_default(cc_serve_config *c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->hbm_budget_bytes = 120ull << 30;
  c->max_batch_graphs = 1024;
  c->compute_streams = 4;  // measured: p99 10 ms at 80 % load against 16-20 ms with 2
  c->smem_max_n = 16384;
}

double cc_serve_now(void) { return ccg::now_s(); }

int cc_serve_create(cc_server **out, int device, const cc_serve_config *cin) {
  using namespace ccg;
  if (!out) return CC_ERR_INVALID;
  *out = nullptr;
  cc_serve_config cfg;
  if (cin) cfg = *cin;
  else cc_serve_config_default(&cfg);
  if (!cfg.max_batch_graphs || !cfg.compute_streams || cfg.compute_streams > 8 ||
      cfg.smem_max_n == 0 || cfg.smem_max_n > 56 * 1024)
    return CC_ERR_INVALID;
  std::unique_ptr<cc_server> h(new cc_server());
  int rc = guard([&] {
    CCG_CUDA(cudaSetDevice(device));
    h->s.reset(new Server(cfg.compute_streams));
    Server &s = *h->s;
    s.device = device;
    s.cfg = cfg;
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    CCG_CUDA(cudaMemPoolCreate(&s.pool, &props));
    uint64_t thr = ~0ull;
    CCG_CUDA(cudaMemPoolSetAttribute(s.pool, cudaMemPoolAttrReleaseThreshold, &thr));
    CCG_CUDA(cudaStreamCreateWithFlags(&s.copy_stream, cudaStreamNonBlocking));
    CCG_CUDA(cudaStreamCreateWithFlags(&s.collect_stream, cudaStreamNonBlocking));
    s.streams.resize(cfg.compute_streams);
    s.desc_dev.resize(cfg.compute_streams);
    s.queue_dev.resize(cfg.compute_streams);
    s.desc_host.resize(cfg.compute_streams, nullptr);
    for (uint32_t i = 0; i < cfg.compute_streams; ++i) {
      CCG_CUDA(cudaStreamCreateWithFlags(&s.streams[i], cudaStreamNonBlocking));
      s.desc_dev[i].alloc(sizeof(GraphDesc) * cfg.max_batch_graphs, s.copy_stream, s.pool);
      s.queue_dev[i].alloc(4, s.copy_stream, s.pool);
      CCG_CUDA(cudaHostAlloc(&s.desc_host[i], sizeof(GraphDesc) * cfg.max_batch_graphs,
                             cudaHostAllocDefault));
    }
    CCG_CUDA(cudaStreamSynchronize(s.copy_stream));
    s.worker = std::thread([&s] { s.loop(); });
  });
  if (rc != CC_OK) return rc;
  *out = h.release();
  return CC_OK;
}

int cc_serve_destroy(cc_server *h) {
  using namespace ccg;
  if (!h) return CC_ERR_INVALID;
  Server &s = *h->s;
  {
    std::lock_guard<std::mutex> lk(s.mu);
    s.stop = true;
  }
  s.cv_worker.notify_all();
  if (s.worker.joinable()) s.worker.join();
  cudaSetDevice(s.device);
  for (auto st : s.streams) cudaStreamSynchronize(st);
  cudaStreamSynchronize(s.copy_stream);
  while (s.inflight.load() > 0) std::this_thread::sleep_for(std::chrono::microseconds(100));
  for (auto &kv : s.reqs) {
    if (kv.second->copied) cudaEventDestroy(kv.second->copied);
  }
  s.reqs.clear();
  s.desc_dev.clear();
  s.queue_dev.clear();
  cudaStreamSynchronize(s.copy_stream);
  for (auto p : s.desc_host)
    if (p) cudaFreeHost(p);
  for (auto st : s.streams) cudaStreamDestroy(st);
  cudaStreamDestroy(s.copy_stream);
  cudaStreamDestroy(s.collect_stream);
  cudaMemPoolDestroy(s.pool);
  delete h;
  return CC_OK;
}

int cc_serve_submit(cc_server *h, const cc_csr *g, uint64_t *ticket) {
  using namespace ccg;
  if (!h || !g || !ticket) return CC_ERR_INVALID;
  if (g->where != CC_HOST || (g->id_bytes != 4 && g->id_bytes != 8) || g->reserved)
    return CC_ERR_INVALID;
  if (g->n == 0 || g->n >= 0xffffffffull) return CC_ERR_UNSUPPORTED;
  if (!g->row_ptr || (g->m_dir && !g->col)) return CC_ERR_INVALID;
  Server &s = *h->s;
  std::unique_ptr<Req> r(new Req());
  r->g = *g;
  r->need = s.bytes_needed(*g);
  if (r->need > s.cfg.hbm_budget_bytes) return CC_ERR_BUSY;
  r->t_submit = now_s();
  r->inject = s.inject_next.exchange(0);
  // the hook schedule of a large graph is host work on the request's own
  // CSR: done here, on the client's thread, it stays off the worker that
  // admits, stages and launches for every client
  if (!s.small(*g)) r->tu = Server::schedule(*g);
  {
    std::lock_guard<std::mutex> lk(s.mu);
    r->id = s.next_id++;
    *ticket = r->id;
    s.waiting.push_back(r.get());
    s.reqs[r->id] = std::move(r);
    s.submitted++;
  }
  s.cv_worker.notify_all();
  return CC_OK;
}

static int collect(cc_server *h, uint64_t ticket, void *labels_out, int *done, double timeout_s,
                   bool block, cc_serve_ticket_info *info) {
  using namespace ccg;
  if (!h || !labels_out) return CC_ERR_INVALID;
  Server &s = *h->s;
  Req *r = nullptr;
  {
    std::unique_lock<std::mutex> lk(s.mu);
    auto it = s.reqs.find(ticket);
    if (it == s.reqs.end()) return CC_ERR_INVALID;
    r = it->second.get();
    if (r->state.load() != kDone) {
      if (!block) {
        if (done) *done = 0;
        return CC_OK;
      }
      auto pred = [&] { return r->state.load() == kDone; };
      if (timeout_s > 0) {
        if (!s.cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
          return CC_ERR_TIMEOUT;
      } else {
        s.cv_done.wait(lk, pred);
      }
    }
  }
  // done: copy the labels and the error word, then retire the request
  int rc = guard([&] {
    CCG_CUDA(cudaSetDevice(s.device));
    const uint64_t n = r->g.n;
    if (r->failed) throw Error(r->fail_status, "request failed before launch");
    if (!r->lab.p) throw Error(CC_ERR_CUDA, "request has no label buffer");
    std::vector<uint32_t> tmp;
    uint32_t *dst = static_cast<uint32_t *>(labels_out);
    if (r->g.id_bytes == 8) {
      tmp.resize(n);
      dst = tmp.data();
    }
    int err = 0;
    CCG_CUDA(cudaMemcpyAsync(dst, r->lab.p, 4 * n, cudaMemcpyDeviceToHost, s.collect_stream));
    CCG_CUDA(cudaMemcpyAsync(&err, r->lab.as<uint32_t>() + n, 4, cudaMemcpyDeviceToHost,
                             s.collect_stream));
    CCG_CUDA(cudaStreamSynchronize(s.collect_stream));
    if (r->g.id_bytes == 8) {
      uint64_t *o = static_cast<uint64_t *>(labels_out);
      for (uint64_t v = 0; v < n; ++v) o[v] = tmp[v];
    }
    if (err) throw Error(CC_ERR_INVALID, "CSR check failed in a served request");
  });
  if (info) {
    info->submit_s = r->t_submit;
    info->admit_s = r->t_admit;
    info->done_s = r->t_done;
    info->batch_id = r->batch_id;
    info->batch_size = r->batch_size;
  }
  std::unique_ptr<Req> retired;
  {
    std::lock_guard<std::mutex> lk(s.mu);
    auto it = s.reqs.find(ticket);
    retired = std::move(it->second);
    s.reqs.erase(it);
    s.used -= retired->need;
    s.collected++;
  }
  // CUDA calls outside the lock: the completion callbacks take it
  if (retired->copied) cudaEventDestroy(retired->copied);
  retired.reset();
  s.cv_worker.notify_all();
  if (done) *done = 1;
  return rc;
}

int cc_serve_poll(cc_server *h, uint64_t ticket, void *labels_out, int *done,
                  cc_serve_ticket_info *info) {
  return collect(h, ticket, labels_out, done, 0.0, false, info);
}

int cc_serve_wait(cc_server *h, uint64_t ticket, void *labels_out, double timeout_s,
                  cc_serve_ticket_info *info) {
  return collect(h, ticket, labels_out, nullptr, timeout_s, true, info);
}

int cc_serve_get_stats(cc_server *h, cc_serve_stats *out) {
  if (!h || !out) return CC_ERR_INVALID;
  ccg::Server &s = *h->s;
  std::lock_guard<std::mutex> lk(s.mu);
  out->submitted = s.submitted;
  out->completed = s.completed;
  out->collected = s.collected;
  out->batches = s.batches;
  out->bytes_in_use = s.used;
  out->peak_bytes_in_use = s.peak;
  out->waiting = s.waiting.size();
  return CC_OK;
}

int cc_serve_debug_fail_next(cc_server *h, int where) {
  if (!h || where < 0 || where > 2) return CC_ERR_INVALID;
  h->s->inject_next = where;
  return CC_OK;
}

}  // extern "C"

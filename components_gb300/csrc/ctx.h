// ctx.h - the context object behind cc_ctx* and the status guard shared by
// the C ABI translation units (api.cu, batch.cu, serve.cu).
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "hostpool.h"
#include "kernels.h"

namespace ccg {
struct BatchCache;  // batch.cu
void batch_cache_free(BatchCache *c);
}  // namespace ccg

struct cc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host-to-device chunks overlapping the tile pass
  bool own_stream = false;
  cudaMemPool_t pool = nullptr;
  int *d_flag = nullptr;
  int *d_err = nullptr;
  int *h_flag = nullptr;  // pinned: [0] round flag, [1] error word at the end of a solve
  uint64_t *d_geo = nullptr;
  int geo_len = 0;
  double geo_beta = -1.0;
  bool prof = false;        // per-kernel CUDA-event timing (CC_PROF_KERNELS)
  bool prof_count = false;  // component count after each solve (CC_PROF_COMPONENTS)
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // solve bracketing events, reused
  std::vector<cudaEvent_t> ev_pool;  // per-kernel profiling events, reused across solves
  ccg::UfTuning uf;  // hook-and-compress schedule (cc_ctx_set_tuning)
  uint32_t round_cap = 0;  // test hook: lower cap on the iterative rounds (0: n + 2)
  int host_reads = 1;      // sampled linking of page-locked host input: 0 copy, 1 read in
                           // place, 2 ids in place and offsets copied (cc_ctx_set_host_reads)
  ccg::UfDecisionCache uf_cache;    // the last device graph's row-sample decisions
  ccg::UfDecisionCache host_cache;  // the last host graph's (streamed input)
  cc_stats stats{};
  cc_stats prof_total{};      // per-kernel sums over the solves since profiling was switched on
  uint64_t prof_solves = 0;
  ccg::BatchCache *batch = nullptr;  // last recorded batch solve (CUDA graph)
  ccg::DevBuf plain_rp;  // per-graph offsets of cc_batch_run_plain (kept for the next call)
  // host threads and page-locked staging of the streamed input (made on first use)
  std::unique_ptr<ccg::HostStager> stager;
};

namespace ccg {

// Last error text of this thread (cc_gpu_strerror).
std::string &last_error();

// The calling thread's context on the current device (made on first use).
cc_ctx *default_context();
// Per-kernel CUDA-event times of c's records into st.kernels (st.nkernels reset).
void collect_kernel_stats(Counters &c, cc_stats &st);

template <class F>
int guard(F &&f) {
  try {
    f();
    return CC_OK;
  } catch (const Error &e) {
    last_error() = e.what();
    return e.status;
  } catch (const std::bad_alloc &) {
    last_error() = "host allocation failed";
    return CC_ERR_OOM;
  } catch (const std::exception &e) {
    last_error() = e.what();
    return CC_ERR_CUDA;
  }
}

// Read the context's error word after the stream drains; throw CC_ERR_INVALID
// when a kernel recorded a bad offset or id.
void throw_on_kernel_error(cc_ctx *C, cudaStream_t s);
// The same check on an error word already copied to the host.
void throw_on_error_word(int e);

}  // namespace ccg

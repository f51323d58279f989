// hostpool.h - host-side helpers of the streamed input path: a small
// persistent pool of host threads and a grow-only page-locked staging buffer.
//
// A host CSR is copied to the device in chunks while the tile pass runs.  The
// host link moves about 200 GB/s, and the row offsets are 8 bytes a vertex;
// rows of fewer than 255 entries are sent as one degree byte instead (the
// device rebuilds the offsets with a prefix sum).  The pool encodes the next
// chunk's degrees while the copy engine moves the current chunk.
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace ccg {

class HostPool {
 public:
  explicit HostPool(unsigned workers) {
    for (unsigned i = 0; i < workers; ++i) th_.emplace_back([this] { loop(); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : th_) t.join();
  }
  HostPool(const HostPool &) = delete;
  HostPool &operator=(const HostPool &) = delete;

  unsigned threads() const { return (unsigned)th_.size() + 1; }

  // f(i) for every i in [0, parts), on the workers and the calling thread;
  // returns when all parts are done.  One caller at a time.
  void run(unsigned parts, const std::function<void(unsigned)> &f) {
    std::unique_lock<std::mutex> l(mu_);
    job_ = &f;
    parts_ = parts;
    next_.store(0);
    busy_ = (unsigned)th_.size();
    ++gen_;
    l.unlock();
    cv_.notify_all();
    work();
    l.lock();
    done_.wait(l, [this] { return busy_ == 0; });
    job_ = nullptr;
  }

 private:
  void work() {
    for (;;) {
      const unsigned i = next_.fetch_add(1);
      if (i >= parts_) return;
      (*job_)(i);
    }
  }
  void loop() {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> l(mu_);
    for (;;) {
      cv_.wait(l, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      l.unlock();
      work();
      l.lock();
      if (--busy_ == 0) done_.notify_one();
    }
  }

  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  const std::function<void(unsigned)> *job_ = nullptr;
  unsigned parts_ = 0;
  std::atomic<unsigned> next_{0};
  unsigned busy_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Page-locked staging memory for the encoded chunks (grow-only) and the pool.
struct HostStager {
  HostPool pool;
  uint8_t *pinned = nullptr;
  size_t cap = 0;
  HostStager() : pool(workers()) {}
  ~HostStager() {
    if (pinned) cudaFreeHost(pinned);
  }
  uint8_t *staging(size_t bytes) {
    if (bytes > cap) {
      if (pinned) cudaFreeHost(pinned);
      pinned = nullptr;
      cap = 0;
      if (cudaHostAlloc((void **)&pinned, bytes, cudaHostAllocDefault) != cudaSuccess) {
        pinned = nullptr;
        return nullptr;
      }
      cap = bytes;
    }
    return pinned;
  }
  // Three quarters of the host cores: the calling thread waits on the device
  // while the workers encode, and a fully subscribed host left a worker
  // descheduled now and then (a solve then waited 30-50 ms for its chunk).
  static unsigned workers() {
    const unsigned hc = std::thread::hardware_concurrency();
    return hc > 2 ? hc * 3 / 4 - 1 : 0;
  }
};

}  // namespace ccg

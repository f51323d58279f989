// Host thread pool of the streamed input path (components_gb300/csrc/hostpool.h):
// every part runs exactly once per run(), runs follow each other, and a pool
// with no workers runs everything on the caller.
#include <atomic>
#include <cstdio>
#include <vector>

#include "hostpool.h"

int main() {
  for (unsigned workers : {0u, 1u, 3u, 15u}) {
    ccg::HostPool pool(workers);
    if (pool.threads() != workers + 1) return 1;
    for (unsigned parts : {0u, 1u, 2u, 7u, 64u, 1000u}) {
      for (int rep = 0; rep < 20; ++rep) {
        std::vector<std::atomic<int>> hits(parts);
        for (auto &h : hits) h.store(0);
        pool.run(parts, [&](unsigned i) { hits[i].fetch_add(1); });
        for (unsigned i = 0; i < parts; ++i)
          if (hits[i].load() != 1) {
            std::printf("workers %u parts %u part %u ran %d times\n", workers, parts, i, hits[i].load());
            return 1;
          }
      }
    }
  }
  std::printf("ok\n");
  return 0;
}

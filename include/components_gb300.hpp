// components_gb300.hpp - the reference's solver classes over the C ABI.
//
// Drop-in for the five solver headers of sebalamm/components
// (lib/components/{exponential_contraction,local_contraction,
// shortcut_propagation,propagation,all_reduce}.h).  The drivers use them as
//
//     ExponentialContraction comp(conf, rank, size);   // app/exp_contraction.cpp:104
//     comp.FindComponents(G, labels);                  // app/exp_contraction.cpp:105
//     comp.GetCommTime(); comp.GetSendVolume(); ...    // app/exp_contraction.cpp:115-129
//
// and the same calls compile against this header.  One process drives one
// GPU: `rank` must be 0 and `size` is the number of virtual ranks, i.e.
// contiguous vertex ranges of the one device-resident graph
// (graph_io.h:308-313).  `labels` receives canonical labels: the minimum
// vertex id of each vertex's component.
//
// Config: any type with the fields of lib/config.h:29-87 (the reference's own
// Config works unchanged).  Graph: any type with the StaticGraph accessors
// GetNumberOfVertices(), ForallLocalVertices(f), ForallNeighbors(v, f) and
// GetGlobalID(v) (static_graph.h), or a ccgpu::HostCsr.
// Errors throw ccgpu::Error carrying the C status code.
#pragma once

#include <cstdint>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cc_gpu.h"

namespace ccgpu {

struct Error : std::runtime_error {
  int status;
  Error(int s, const char *msg) : std::runtime_error(std::string("libccgpu: ") + msg), status(s) {}
};

inline void check(int status) {
  if (status != CC_OK) throw Error(status, cc_gpu_strerror(status));
}

// A host CSR that is passed to the library without an adapter pass.
struct HostCsr {
  std::vector<uint64_t> row_ptr;  // n+1
  std::vector<uint64_t> col;      // symmetric adjacency, 64-bit ids
  uint64_t GetNumberOfVertices() const { return row_ptr.empty() ? 0 : row_ptr.size() - 1; }
};

template <class ConfigT>
cc_config to_cc_config(const ConfigT &conf) {
  cc_config c;
  cc_config_default(&c);
  c.beta = conf.beta;
  c.seq = (uint32_t)conf.sequential_limit;
  c.prop_iterations = (uint32_t)conf.prop_iterations;
  c.number_of_hitters = (uint32_t)conf.number_of_hitters;
  c.degree_threshold = (uint32_t)conf.degree_threshold;
  c.degree_limit = (uint32_t)conf.degree_limit;
  c.hd_sf = (float)conf.neighborhood_sampling_factor;
  c.fixed_seq = conf.fixed_limit;
  c.contraction = conf.use_contraction;
  c.direct = conf.direct_contraction;
  c.single = conf.single_level_contraction;
  c.bfs = conf.use_bfs;
  c.replicate = conf.replicate_high_degree;
  c.regular = conf.use_regular;
  c.overalloc = conf.overallocate;
  c.verbose = conf.print_verbose;
  return c;
}

template <cc_algo ALGO>
class Solver {
 public:
  template <class ConfigT>
  Solver(const ConfigT &conf, int rank, int size)
      : cfg_(to_cc_config(conf)), seed_((uint64_t)(int64_t)conf.seed), size_(size) {
    if (rank != 0) throw Error(CC_ERR_INVALID, "one process drives one GPU: rank must be 0");
    if (size < 1) throw Error(CC_ERR_INVALID, "size must be >= 1");
  }
  virtual ~Solver() = default;

  // CSR already in hand: no adapter pass.
  void FindComponents(const HostCsr &g, std::vector<unsigned long long> &labels) {
    run_csr(g, labels);
  }
  void FindComponents(HostCsr &g, std::vector<unsigned long long> &labels) { run_csr(g, labels); }

  // Reference graph types: the CSR is read through the StaticGraph accessors.
  template <class GraphType>
  void FindComponents(GraphType &g, std::vector<unsigned long long> &labels) {
    HostCsr h;
    const uint64_t n = g.GetNumberOfVertices();
    h.row_ptr.assign(n + 1, 0);
    h.col.reserve(2 * n);
    std::vector<uint64_t> local;
    local.reserve(n);
    g.ForallLocalVertices([&](const unsigned long long v) {
      local.push_back(v);
      g.ForallNeighbors(v, [&](const unsigned long long w) { h.col.push_back(g.GetGlobalID(w)); });
      h.row_ptr[g.GetGlobalID(v) + 1] = h.col.size();
    });
    for (uint64_t v = 0; v < n; ++v)
      if (h.row_ptr[v + 1] < h.row_ptr[v]) h.row_ptr[v + 1] = h.row_ptr[v];
    std::vector<unsigned long long> out(n);
    run_csr(h, out);
    if (labels.size() < n) labels.resize(n);
    for (uint64_t v : local) labels[v] = out[g.GetGlobalID(v)];
  }

  float GetCommTime() { return 0.f; }
  unsigned long long GetSendVolume() { return 0; }
  unsigned long long GetReceiveVolume() { return 0; }
  const cc_stats &GetStats() const { return stats_; }

 private:
  void run_csr(const HostCsr &g, std::vector<unsigned long long> &labels) {
    const uint64_t n = g.GetNumberOfVertices();
    if (labels.size() < n) labels.resize(n);
    cc_csr c{n, (uint64_t)g.col.size(), g.row_ptr.data(), g.col.data(), 8, (uint32_t)size_,
             CC_HOST, 0};
    check(cc_gpu_run(&c, ALGO, &cfg_, seed_, labels.data()));
    check(cc_gpu_stats(&stats_));
  }

  cc_config cfg_;
  uint64_t seed_;
  int size_;
  cc_stats stats_{};
};

using ExponentialContraction = Solver<CC_EXP>;
using LocalContraction = Solver<CC_LOCAL>;
using ShortcutPropagation = Solver<CC_SHORTCUTS>;
using Propagation = Solver<CC_LABELS>;
template <class GraphType>
class AllReduce : public Solver<CC_ALLREDUCE> {
 public:
  using Solver<CC_ALLREDUCE>::Solver;
};

// The reference's StaticGraph::OutputComponents (static_graph.h:504-591) for
// the labels of a FindComponents call: the component-size distribution, in
// ascending size, and the number of components with more than one vertex,
// printed in the reference's format.  The counting runs on the device.
inline uint64_t OutputComponents(const std::vector<unsigned long long> &labels,
                                 std::ostream &os = std::cout) {
  const uint64_t n = labels.size();
  uint64_t cap = 2;
  while (cap * cap < 2 * n) cap *= 2;
  cap += 2;
  std::vector<uint64_t> pairs(2 * cap);
  uint64_t k = 0, num = 0;
  check(cc_component_sizes(nullptr, labels.data(), 8, CC_HOST, n, pairs.data(), cap, &k, &num));
  os << "COMPONENTS [ ";
  for (uint64_t i = 0; i < k && i < cap; ++i)
    os << "size=" << pairs[2 * i] << " (num=" << pairs[2 * i + 1] << ") ";
  os << "]" << std::endl;
  os << "NUM COMPONENTS " << num << std::endl;
  return num;
}

}  // namespace ccgpu

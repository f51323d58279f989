// Driver-shaped use of include/components_gb300.hpp: the calls of
// app/exp_contraction.cpp:95-129 against a graph type that offers the
// StaticGraph accessors the header reads.  Prints one line per solver:
// "<name> <label_0> <label_1> ..." for the graph given on stdin
// ("n m" then m undirected edges "u w"), then the component summary lines
// "COMPONENTS [ size=.. (num=..) ... ]" and "NUM COMPONENTS k".
#include <cstdio>
#include <functional>
#include <vector>

#include "components_gb300.hpp"

struct Config {  // the fields of lib/config.h that the header reads
  int seed = 1;
  bool print_verbose = false;
  unsigned long long degree_limit = 100;
  bool replicate_high_degree = false;
  unsigned long long sequential_limit = 1;
  bool fixed_limit = false;
  unsigned int prop_iterations = 3;
  double beta = 0.1;
  bool use_bfs = false, use_regular = false, overallocate = false;
  bool use_contraction = false, direct_contraction = false, single_level_contraction = false;
  unsigned long long number_of_hitters = 0, degree_threshold = 16;
  float neighborhood_sampling_factor = 0.5f;
};

struct TinyStaticGraph {  // StaticGraph accessor names, one rank
  std::vector<std::vector<unsigned long long>> adj;
  unsigned long long GetNumberOfVertices() const { return adj.size(); }
  unsigned long long GetVertexVectorSize() const { return adj.size(); }
  unsigned long long GetGlobalID(unsigned long long v) const { return v; }
  void ForallLocalVertices(const std::function<void(unsigned long long)> &f) {
    for (unsigned long long v = 0; v < adj.size(); ++v) f(v);
  }
  void ForallNeighbors(unsigned long long v, const std::function<void(unsigned long long)> &f) {
    for (auto w : adj[v]) f(w);
  }
};

template <class Solver>
void run(const char *name, Config conf, int size, TinyStaticGraph &G) {
  std::vector<unsigned long long> labels(G.GetVertexVectorSize(), 0);
  G.ForallLocalVertices([&](unsigned long long v) { labels[v] = G.GetGlobalID(v); });
  Solver comp(conf, 0, size);
  comp.FindComponents(G, labels);
  std::printf("%s", name);
  for (auto l : labels) std::printf(" %llu", l);
  std::printf(" comm=%g send=%llu recv=%llu\n", comp.GetCommTime(), comp.GetSendVolume(),
              comp.GetReceiveVolume());
}

int main() {
  unsigned long long n, m;
  if (std::scanf("%llu %llu", &n, &m) != 2) return 2;
  TinyStaticGraph G;
  G.adj.resize(n);
  for (unsigned long long i = 0; i < m; ++i) {
    unsigned long long u, w;
    if (std::scanf("%llu %llu", &u, &w) != 2) return 2;
    G.adj[u].push_back(w);
    G.adj[w].push_back(u);
  }
  Config conf;
  conf.seed = 1001;
  conf.sequential_limit = 0;
  try {
    run<ccgpu::ExponentialContraction>("exp", conf, 3, G);
    run<ccgpu::LocalContraction>("local", conf, 3, G);
    run<ccgpu::ShortcutPropagation>("shortcuts", conf, 3, G);
    run<ccgpu::Propagation>("labels", conf, 3, G);
    run<ccgpu::AllReduce<TinyStaticGraph>>("allreduce", conf, 3, G);
    // the drivers' closing summary (StaticGraph::OutputComponents)
    std::vector<unsigned long long> labels(G.GetVertexVectorSize(), 0);
    ccgpu::ExponentialContraction comp(conf, 0, 1);
    comp.FindComponents(G, labels);
    ccgpu::OutputComponents(labels);
  } catch (const ccgpu::Error &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}

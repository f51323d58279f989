// The drivers' graph input through include/components_gb300_io.hpp: prints
// "n m_dir", then the row offsets, then the ids, for
//   io_main file|edgefile|binary <path>   or   io_main gen <model> <n> <m> <p> <d> <gamma> <seed>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "components_gb300_io.hpp"

struct Config {  // the input fields of lib/config.h
  std::string input_type = "null", input_file = "null", gen = "null";
  unsigned long long gen_n = 0, gen_m = 0;
  float gen_p = 1.0f, gen_d = 16.0f, gen_gamma = 2.2f;
  bool gen_periodic = false;
  int seed = 1;
};

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  Config conf;
  if (std::string(argv[1]) == "gen") {
    if (argc < 9) return 2;
    conf.gen = argv[2];
    conf.gen_n = std::strtoull(argv[3], nullptr, 10);
    conf.gen_m = std::strtoull(argv[4], nullptr, 10);
    conf.gen_p = std::strtof(argv[5], nullptr);
    conf.gen_d = std::strtof(argv[6], nullptr);
    conf.gen_gamma = std::strtof(argv[7], nullptr);
    conf.seed = std::atoi(argv[8]);
  } else {
    conf.input_type = argv[1];
    conf.input_file = argv[2];
  }
  try {
    const ccgpu::HostCsr g = ccgpu::LoadGraph(conf);
    std::printf("%llu %llu\n", (unsigned long long)g.GetNumberOfVertices(), (unsigned long long)g.col.size());
    for (auto x : g.row_ptr) std::printf("%llu ", (unsigned long long)x);
    std::printf("\n");
    for (auto x : g.col) std::printf("%llu ", (unsigned long long)x);
    std::printf("\n");
  } catch (const ccgpu::Error &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}

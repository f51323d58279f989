// components_gb300_io.hpp - the drivers' graph input over libccgen.
//
// Drop-in for IOUtility::LoadGraph (lib/io/io_utils.h:33-56) as the five
// drivers of app/ call it, for one process driving one GPU:
//
//     ccgpu::HostCsr G = ccgpu::LoadGraph(conf);   // instead of IOUtility::LoadGraph(G, conf, rank, size)
//     ccgpu::ExponentialContraction comp(conf, 0, size);
//     comp.FindComponents(G, labels);
//
// `-input file|edgefile|binary -in <path>` reads the METIS text, sorted edge
// or sorted binary file; otherwise `-gen gnm_undirected|grid_2d|rhg` builds the
// graph with the seeded generators of cc_gen.h.  Config: any type with the
// fields of lib/config.h (input_type, input_file, gen, gen_n, gen_m, gen_p,
// gen_d, gen_gamma, gen_periodic, seed).  Link with -lccgen.  Errors throw
// ccgpu::Error.
#pragma once

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "cc_gen.h"
#include "components_gb300.hpp"

namespace ccgpu {

inline HostCsr to_host_csr(cc_host_graph &hg) {
  HostCsr g;
  g.row_ptr.assign(hg.row_ptr, hg.row_ptr + hg.n + 1);
  g.col.resize(hg.m_dir);
  const uint32_t *c32 = static_cast<const uint32_t *>(hg.col);
  const uint64_t *c64 = static_cast<const uint64_t *>(hg.col);
  for (uint64_t e = 0; e < hg.m_dir; ++e) g.col[e] = hg.id_bytes == 8 ? c64[e] : c32[e];
  cc_host_graph_free(&hg);
  return g;
}

template <class ConfigT>
HostCsr LoadGraph(const ConfigT &conf) {
  cc_host_graph hg;
  std::memset(&hg, 0, sizeof(hg));
  const std::string type(conf.input_type), gen(conf.gen);
  const char *path = conf.input_file.c_str();
  int rc = CC_ERR_INVALID;
  if (type == "file") {
    rc = cc_read_metis(path, 8, &hg);
  } else if (type == "edgefile") {
    rc = cc_read_edge_list(path, 8, &hg);
  } else if (type == "binary") {
    rc = cc_read_binary_edges(path, 8, &hg);
  } else if (type == "partition") {
    throw Error(CC_ERR_UNSUPPORTED, "-input partition (one edge file per rank) is not read on one device");
  } else if (gen == "gnm_undirected") {
    rc = cc_gen_gnm(conf.gen_n, conf.gen_m, (uint64_t)conf.seed, 8, &hg);
  } else if (gen == "grid_2d") {
    if (conf.gen_periodic) throw Error(CC_ERR_UNSUPPORTED, "-periodic grids are not generated");
    rc = cc_gen_grid(conf.gen_n, conf.gen_m, conf.gen_p, (uint64_t)conf.seed, 8, &hg);
  } else if (gen == "rhg") {
    rc = cc_gen_rhg(conf.gen_n, conf.gen_d, conf.gen_gamma, (uint64_t)conf.seed, 8, &hg);
  } else {
    throw Error(CC_ERR_UNSUPPORTED, "I/O type not supported (-input file|edgefile|binary, or -gen "
                                    "gnm_undirected|grid_2d|rhg)");
  }
  check(rc);
  return to_host_csr(hg);
}

}  // namespace ccgpu

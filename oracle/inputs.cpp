/*
 * inputs.cpp - seeded input graphs for the oracle's own runs.
 *
 * TEST INFRASTRUCTURE ONLY.  The CPU baseline of the benchmark and its
 * reference arm must solve the very graph the GPU solves, without loading the
 * GPU library or libccgen.  libccoracle.so is therefore linked with the
 * library's generator source (components_gb300/csrc/gen.cpp, compiled with
 * hidden symbols), and this file exports its generators under or_* names.
 * The generators only build inputs; nothing here computes components.
 */
#include "../include/cc_gen.h"

#define OR_EXPORT extern "C" __attribute__((visibility("default")))

OR_EXPORT int or_gen_gnm(uint64_t n, uint64_t m, uint64_t seed, uint32_t id_bytes,
                         cc_host_graph *out) {
  return cc_gen_gnm(n, m, seed, id_bytes, out);
}

OR_EXPORT int or_gen_grid(uint64_t X, uint64_t Y, double p, uint64_t seed, uint32_t id_bytes,
                          cc_host_graph *out) {
  return cc_gen_grid(X, Y, p, seed, id_bytes, out);
}

OR_EXPORT int or_gen_rhg(uint64_t n, double avg_deg, double gamma, uint64_t seed,
                         uint32_t id_bytes, cc_host_graph *out) {
  return cc_gen_rhg(n, avg_deg, gamma, seed, id_bytes, out);
}

OR_EXPORT void or_graph_free(cc_host_graph *g) { cc_host_graph_free(g); }

// gen.cpp - seeded synthetic graph generators (host C++, libccgen.so).
//
// Stand-ins for the KaGen generators the reference drivers call through
// IOUtility::LoadGraph (lib/io/io_utils.h:59-83).  All randomness comes from a
// SplitMix64 hash of (seed, index, stream), so the same arguments give the
// same graph on every host and for every thread count.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/cc_gen.h"
#include "../../include/cc_gpu.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
inline uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
  return mix64(mix64(mix64(seed) ^ a) ^ (b * 0xd6e8feb86659fd93ull));
}
// uniform integer in [0, n) from the high word (n < 2^32)
inline uint64_t below(uint64_t h, uint64_t n) { return ((h >> 32) * n) >> 32; }
// uniform double in [0, 1)
inline double unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

void radix_u64(std::vector<uint64_t> &a, int bits) {
  std::vector<uint64_t> tmp(a.size());
  std::vector<uint64_t> cnt(65536);
  uint64_t *src = a.data(), *dst = tmp.data();
  const uint64_t n = a.size();
  for (int sh = 0; sh < bits; sh += 16) {
    std::fill(cnt.begin(), cnt.end(), 0);
    for (uint64_t i = 0; i < n; ++i) cnt[(src[i] >> sh) & 0xffff]++;
    uint64_t run = 0;
    for (auto &c : cnt) {
      uint64_t t = c;
      c = run;
      run += t;
    }
    for (uint64_t i = 0; i < n; ++i) dst[cnt[(src[i] >> sh) & 0xffff]++] = src[i];
    std::swap(src, dst);
  }
  if (src != a.data()) std::memcpy(a.data(), src, 8 * n);
}

int bits_for(uint64_t x) {
  int b = 1;
  while (b < 64 && (1ull << b) < x) ++b;
  return b;
}

bool alloc_graph(cc_host_graph *out, uint64_t n, uint64_t m, uint32_t idb) {
  out->n = n;
  out->m_dir = m;
  out->id_bytes = idb;
  out->pad_ = 0;
  out->row_ptr = static_cast<uint64_t *>(std::malloc(8 * (n + 1)));
  out->col = std::malloc((size_t)idb * (m ? m : 1));
  if (!out->row_ptr || !out->col) {
    std::free(out->row_ptr);
    std::free(out->col);
    out->row_ptr = nullptr;
    out->col = nullptr;
    return false;
  }
  return true;
}

inline void put_id(cc_host_graph *g, uint64_t e, uint64_t id) {
  if (g->id_bytes == 8) static_cast<uint64_t *>(g->col)[e] = id;
  else static_cast<uint32_t *>(g->col)[e] = (uint32_t)id;
}

// CSR from sorted, deduplicated directed keys (src << b) | dst.
int csr_from_keys(const std::vector<uint64_t> &keys, int b, uint64_t n, uint32_t idb,
                  cc_host_graph *out) {
  if (!alloc_graph(out, n, keys.size(), idb)) return CC_ERR_OOM;
  std::memset(out->row_ptr, 0, 8 * (n + 1));
  const uint64_t mask = (1ull << b) - 1;
  for (uint64_t i = 0; i < keys.size(); ++i) {
    out->row_ptr[(keys[i] >> b) + 1]++;
    put_id(out, i, keys[i] & mask);
  }
  for (uint64_t v = 0; v < n; ++v) out->row_ptr[v + 1] += out->row_ptr[v];
  return CC_OK;
}

}  // namespace

extern "C" {

int cc_gen_gnm(uint64_t n, uint64_t m, uint64_t seed, uint32_t id_bytes, cc_host_graph *out) {
  if (!out || (id_bytes != 4 && id_bytes != 8) || n == 0 || n >= (1ull << 32))
    return CC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  const int b = bits_for(n);
  std::vector<uint64_t> keys(2 * m);
  const uint64_t none = ~0ull;
  long long i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < (long long)m; ++i) {
    uint64_t u = below(hash3(seed, (uint64_t)i, 1), n);
    uint64_t w = below(hash3(seed, (uint64_t)i, 2), n);
    if (u == w) {
      keys[2 * i] = keys[2 * i + 1] = none;  // self-loop dropped
    } else {
      keys[2 * i] = (u << b) | w;
      keys[2 * i + 1] = (w << b) | u;
    }
  }
  keys.erase(std::remove(keys.begin(), keys.end(), none), keys.end());
  radix_u64(keys, 2 * b);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());  // duplicates dropped
  return csr_from_keys(keys, b, n, id_bytes, out);
}

int cc_gen_grid(uint64_t X, uint64_t Y, double p, uint64_t seed, uint32_t id_bytes,
                cc_host_graph *out) {
  if (!out || (id_bytes != 4 && id_bytes != 8) || X == 0 || Y == 0) return CC_ERR_INVALID;
  const uint64_t n = X * Y;
  if (n >= (1ull << 32) && id_bytes == 4) return CC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  // edge kept iff hash < thr; thr = p * 2^64 (p >= 1: all, p <= 0: none)
  const bool all = p >= 1.0, none = p <= 0.0;
  const uint64_t thr = (all || none) ? 0 : (uint64_t)std::ldexp(p, 64);
  auto right = [&](uint64_t v) {  // edge v -- v+1 (same row)
    return (v % X) + 1 < X && (all || (!none && hash3(seed, v, 0) < thr));
  };
  auto down = [&](uint64_t v) {  // edge v -- v+X
    return v / X + 1 < Y && (all || (!none && hash3(seed, v, 1) < thr));
  };
  std::vector<uint64_t> deg(n + 1, 0);
  long long y;
#pragma omp parallel for schedule(static)
  for (y = 0; y < (long long)Y; ++y)
    for (uint64_t x = 0; x < X; ++x) {
      uint64_t v = (uint64_t)y * X + x;
      uint64_t d = 0;
      if (y > 0 && down(v - X)) ++d;
      if (x > 0 && right(v - 1)) ++d;
      if (right(v)) ++d;
      if (down(v)) ++d;
      deg[v] = d;
    }
  uint64_t run = 0;
  for (uint64_t v = 0; v < n; ++v) {
    uint64_t d = deg[v];
    deg[v] = run;
    run += d;
  }
  deg[n] = run;
  if (!alloc_graph(out, n, run, id_bytes)) return CC_ERR_OOM;
  std::memcpy(out->row_ptr, deg.data(), 8 * (n + 1));
#pragma omp parallel for schedule(static)
  for (y = 0; y < (long long)Y; ++y)
    for (uint64_t x = 0; x < X; ++x) {
      uint64_t v = (uint64_t)y * X + x, e = out->row_ptr[v];
      if (y > 0 && down(v - X)) put_id(out, e++, v - X);
      if (x > 0 && right(v - 1)) put_id(out, e++, v - 1);
      if (right(v)) put_id(out, e++, v + 1);
      if (down(v)) put_id(out, e++, v + X);
    }
  return CC_OK;
}

int cc_gen_rhg(uint64_t, double, double, uint64_t, uint32_t, cc_host_graph *out) {
  if (out) std::memset(out, 0, sizeof(*out));
  return CC_ERR_UNSUPPORTED;
}

void cc_host_graph_free(cc_host_graph *g) {
  if (!g) return;
  std::free(g->row_ptr);
  std::free(g->col);
  g->row_ptr = nullptr;
  g->col = nullptr;
}

int cc_gen_batch(uint32_t k, double log2_nmin, double log2_nmax, double dmin, double dmax,
                 uint64_t seed, cc_host_batch *out) {
  if (!out || log2_nmin < 0 || log2_nmax < log2_nmin || log2_nmax > 31 || dmin < 0 || dmax < dmin)
    return CC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::vector<uint64_t> n(k), m(k);
  for (uint32_t i = 0; i < k; ++i) {
    double ln = log2_nmin + (log2_nmax - log2_nmin) * unit(hash3(seed, i, 11));
    n[i] = std::max<uint64_t>(1, (uint64_t)std::llround(std::exp2(ln)));
    double d = dmin + (dmax - dmin) * unit(hash3(seed, i, 12));
    m[i] = (uint64_t)std::llround((double)n[i] * d / 2.0);
  }
  std::vector<cc_host_graph> parts(k);
  int bad = 0;
  long long i;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
  for (i = 0; i < (long long)k; ++i) {
    // one graph: the G(n, m) generator on its own seed, single-threaded here
    const uint64_t gs = hash3(seed, (uint64_t)i, 13), gn = n[i], gm = m[i];
    const int b = bits_for(gn);
    std::vector<uint64_t> keys;
    keys.reserve(2 * gm);
    for (uint64_t j = 0; j < gm; ++j) {
      uint64_t u = below(hash3(gs, j, 1), gn), w = below(hash3(gs, j, 2), gn);
      if (u == w) continue;
      keys.push_back((u << b) | w);
      keys.push_back((w << b) | u);
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    if (csr_from_keys(keys, b, gn, 4, &parts[i]) != CC_OK) bad |= 1;
  }
  if (bad) {
    for (auto &p : parts) cc_host_graph_free(&p);
    return CC_ERR_OOM;
  }
  out->k = k;
  out->voff = static_cast<uint64_t *>(std::malloc(8 * (k + 1)));
  std::vector<uint64_t> eoff(k + 1, 0);
  out->voff[0] = 0;
  for (uint32_t j = 0; j < k; ++j) {
    out->voff[j + 1] = out->voff[j] + parts[j].n;
    eoff[j + 1] = eoff[j] + parts[j].m_dir;
  }
  out->total_n = out->voff[k];
  out->total_m = eoff[k];
  out->row_ptr = static_cast<uint64_t *>(std::malloc(8 * (out->total_n + 1)));
  out->col = static_cast<uint32_t *>(std::malloc(4 * (out->total_m ? out->total_m : 1)));
  if (!out->voff || !out->row_ptr || !out->col) {
    for (auto &p : parts) cc_host_graph_free(&p);
    cc_host_batch_free(out);
    return CC_ERR_OOM;
  }
#pragma omp parallel for schedule(dynamic, 4)
  for (i = 0; i < (long long)k; ++i) {
    const cc_host_graph &p = parts[i];
    for (uint64_t v = 0; v < p.n; ++v) out->row_ptr[out->voff[i] + v] = eoff[i] + p.row_ptr[v];
    if (p.m_dir) std::memcpy(out->col + eoff[i], p.col, 4 * p.m_dir);
  }
  out->row_ptr[out->total_n] = out->total_m;
  for (auto &p : parts) cc_host_graph_free(&p);
  return CC_OK;
}

void cc_host_batch_free(cc_host_batch *b) {
  if (!b) return;
  std::free(b->voff);
  std::free(b->row_ptr);
  std::free(b->col);
  b->voff = b->row_ptr = nullptr;
  b->col = nullptr;
}

}  // extern "C"

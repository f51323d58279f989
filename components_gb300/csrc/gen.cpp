// gen.cpp - seeded synthetic graph generators (host C++, libccgen.so).
//
// Stand-ins for the KaGen generators the reference drivers call through
// IOUtility::LoadGraph (lib/io/io_utils.h:59-83).  All randomness comes from a
// SplitMix64 hash of (seed, index, stream), so the same arguments give the
// same graph on every host and for every thread count.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/cc_gen.h"
#include "../../include/cc_gpu.h"
#include "rhg.h"

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

}  // extern "C"

// ---- random hyperbolic graphs (threshold model) ------------------------------
// The model, the exact edge test and the candidate search are in rhg.h, shared
// with the device generator; here the disk radius for a target average degree
// and the host's neighbour search.
namespace {

// Sorted keys, points and per-band cell tables of one graph.
struct RhgLayout {
  std::vector<rhg::Point> pt;                 // by vertex id (angular order)
  std::vector<std::vector<uint32_t>> band;    // vertex ids per band, ascending
  std::vector<std::vector<uint64_t>> cell;    // per band: 2^L + 1 cell starts into band[b]
  std::vector<int> L;
};

void rhg_layout(const rhg::Params &P, RhgLayout &lay) {
  const uint64_t n = P.n;
  std::vector<uint64_t> key(n);
  long long i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < (long long)n; ++i) key[i] = rhg::angle_key(P, (uint64_t)i);
  radix_u64(key, 64);
  lay.pt.resize(n);
#pragma omp parallel for schedule(static)
  for (i = 0; i < (long long)n; ++i) lay.pt[i] = rhg::point(P, key[i]);
  std::vector<uint64_t>().swap(key);
  lay.band.assign(P.nb, {});
  for (uint64_t v = 0; v < n; ++v) lay.band[lay.pt[v].band].push_back((uint32_t)v);
  lay.cell.assign(P.nb, {});
  lay.L.assign(P.nb, 0);
  for (int b = 0; b < P.nb; ++b) {
    const int L = rhg::cell_bits(lay.band[b].size());
    lay.L[b] = L;
    std::vector<uint64_t> &c = lay.cell[b];
    c.assign((1ull << L) + 1, 0);
    for (uint32_t v : lay.band[b]) c[rhg::cell_of(lay.pt[v].phi, L) + 1]++;
    for (uint64_t k = 0; k < (1ull << L); ++k) c[k + 1] += c[k];
  }
}

// Every neighbour of v, appended to out (unsorted: band by band).
void rhg_neighbours(const rhg::Params &P, const RhgLayout &lay, uint64_t v,
                    std::vector<uint32_t> &out) {
  const rhg::Point &pv = lay.pt[v];
  const double inv_s = pv.s > 0.0 ? 1.0 / pv.s : 0.0;
  for (int b = 0; b < P.nb; ++b) {
    const std::vector<uint32_t> &bp = lay.band[b];
    if (bp.empty()) continue;
    uint64_t half = 0;
    const int L = lay.L[b];
    const bool win = L > 0 && rhg::window(P, pv, b, inv_s, &half);
    auto scan = [&](uint64_t k0, uint64_t k1) {
      for (uint64_t k = k0; k < k1; ++k) {
        const uint32_t w = bp[k];
        if (w == v) continue;
        const rhg::Point &pw = lay.pt[w];
        if (win && pw.phi - (pv.phi - half) > 2 * half) continue;
        if (rhg::adjacent(P, pv, pw)) out.push_back(w);
      }
    };
    if (!win) {
      scan(0, bp.size());
      continue;
    }
    const uint64_t lo = pv.phi - half, hi = pv.phi + half;
    const uint64_t c0 = rhg::cell_of(lo, L), c1 = rhg::cell_of(hi, L);
    const std::vector<uint64_t> &c = lay.cell[b];
    if (lo > pv.phi || hi < pv.phi) {  // the window crosses angle 0
      scan(c[c0], bp.size());
      scan(0, c[c1 + 1]);
    } else {
      scan(c[c0], c[c1 + 1]);
    }
  }
}

}  // namespace

extern "C" {

int cc_gen_rhg(uint64_t n, double avg_deg, double gamma, uint64_t seed, uint32_t id_bytes,
               cc_host_graph *out) {
  if (!out || (id_bytes != 4 && id_bytes != 8)) return CC_ERR_INVALID;
  rhg::Params P;
  int st = rhg::make_params(n, avg_deg, gamma, seed, &P);
  if (st != CC_OK) return st;
  std::memset(out, 0, sizeof(*out));
  RhgLayout lay;
  rhg_layout(P, lay);
  // neighbours of every point, threads over contiguous point ranges
  int T = 1;
#ifdef _OPENMP
  T = omp_get_max_threads();
#endif
  std::vector<std::vector<uint32_t>> nbr(T);
  std::vector<uint64_t> deg(n + 1, 0);
#pragma omp parallel num_threads(T)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    const uint64_t lo = n * (uint64_t)t / T, hi = n * (uint64_t)(t + 1) / T;
    std::vector<uint32_t> &out_t = nbr[t];
    out_t.reserve((size_t)((hi - lo) * avg_deg * 1.1));
    for (uint64_t v = lo; v < hi; ++v) {
      const uint64_t before = out_t.size();
      rhg_neighbours(P, lay, v, out_t);
      std::sort(out_t.begin() + before, out_t.end());
      deg[v + 1] = out_t.size() - before;
    }
  }
  for (uint64_t v = 0; v < n; ++v) deg[v + 1] += deg[v];
  if (!alloc_graph(out, n, deg[n], id_bytes)) return CC_ERR_OOM;
  std::memcpy(out->row_ptr, deg.data(), 8 * (n + 1));
#pragma omp parallel num_threads(T)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    const uint64_t lo = n * (uint64_t)t / T;
    uint64_t e = deg[lo];
    for (uint32_t w : nbr[t]) put_id(out, e++, w);
  }
  return CC_OK;
}

double cc_gen_rhg_radius(uint64_t n, double avg_deg, double gamma) {
  rhg::Params P;
  return rhg::make_params(n, avg_deg, gamma, 1, &P) == CC_OK ? P.R : -1.0;
}

uint64_t cc_gen_rhg_verify(uint64_t n, double avg_deg, double gamma, uint64_t seed,
                           const cc_host_graph *g) {
  rhg::Params P;
  if (!g || g->n != n || rhg::make_params(n, avg_deg, gamma, seed, &P) != CC_OK) return ~0ull;
  std::vector<uint64_t> key(n);
  for (uint64_t i = 0; i < n; ++i) key[i] = rhg::angle_key(P, i);
  std::sort(key.begin(), key.end());
  std::vector<rhg::Point> pt(n);
  for (uint64_t i = 0; i < n; ++i) pt[i] = rhg::point(P, key[i]);
  auto id = [&](uint64_t e) -> uint64_t {
    return g->id_bytes == 8 ? static_cast<const uint64_t *>(g->col)[e]
                            : static_cast<const uint32_t *>(g->col)[e];
  };
  uint64_t bad = 0;
  long long v;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : bad)
  for (v = 0; v < (long long)n; ++v) {
    uint64_t e = g->row_ptr[v];
    const uint64_t end = g->row_ptr[v + 1];
    for (uint64_t w = 0; w < n; ++w) {
      const bool want = w != (uint64_t)v && rhg::adjacent(P, pt[v], pt[w]);
      const bool have = e < end && id(e) == w;
      if (have) ++e;
      if (want != have) ++bad;
    }
    if (e != end) bad += end - e;
  }
  return bad;
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

// ---- input files (the reference's GraphIO readers, lib/io/graph_io.h) --------
// Every reader collects the undirected edges, drops self-loops and repeats,
// and builds the symmetric CSR with sorted rows, as the generators do.
namespace {

bool slurp(const char *path, std::vector<char> &buf) {
  FILE *f = path ? std::fopen(path, "rb") : nullptr;
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (len < 0) {
    std::fclose(f);
    return false;
  }
  buf.resize((size_t)len + 1);
  const size_t got = len ? std::fread(buf.data(), 1, (size_t)len, f) : 0;
  std::fclose(f);
  buf.resize(got);
  buf.push_back('\n');  // every line ends with a newline
  return got == (size_t)len;
}

// Unsigned decimal at p (spaces and tabs skipped first); false at the end of
// the line.
bool next_uint(const char *&p, const char *eol, uint64_t &v) {
  while (p < eol && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
  if (p >= eol || *p < '0' || *p > '9') return false;
  v = 0;
  while (p < eol && *p >= '0' && *p <= '9') v = 10 * v + (uint64_t)(*p++ - '0');
  return true;
}

// CSR of the undirected edges (u, w) (0-based, below n) collected as keys.
int csr_from_edges(std::vector<uint64_t> &keys, uint64_t n, uint32_t idb, cc_host_graph *out) {
  const int b = bits_for(n);
  radix_u64(keys, 2 * b);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  return csr_from_keys(keys, b, n, idb, out);
}
void add_edge(std::vector<uint64_t> &keys, int b, uint64_t u, uint64_t w) {
  if (u == w) return;
  keys.push_back((u << b) | w);
  keys.push_back((w << b) | u);
}

}  // namespace

extern "C" {

// METIS text (ReadMETISFile, graph_io.h:281-382): '%' comment lines, a header
// "n m ..." (m is not trusted), then one line per vertex with its 1-based
// neighbours.
int cc_read_metis(const char *path, uint32_t id_bytes, cc_host_graph *out) {
  if (!out || (id_bytes != 4 && id_bytes != 8)) return CC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::vector<char> buf;
  if (!slurp(path, buf)) return CC_ERR_INVALID;
  const char *p = buf.data(), *end = buf.data() + buf.size();
  auto line = [&](const char *&a, const char *&e) {  // next line that is not a comment
    while (p < end) {
      a = p;
      e = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
      p = e + 1;
      if (*a != '%') return true;
    }
    return false;
  };
  const char *a, *e;
  uint64_t n = 0, m_hdr = 0;
  if (!line(a, e) || !next_uint(a, e, n) || !next_uint(a, e, m_hdr)) return CC_ERR_INVALID;
  if (n == 0 || n >= (1ull << 32) || (id_bytes == 4 && n >= 0xffffffffull)) return CC_ERR_INVALID;
  const int b = bits_for(n);
  std::vector<uint64_t> keys;
  keys.reserve(2 * m_hdr + 16);
  for (uint64_t v = 0; v < n; ++v) {
    if (!line(a, e)) break;  // missing trailing lines: isolated vertices
    uint64_t t;
    while (next_uint(a, e, t)) {
      if (t == 0 || t > n) return CC_ERR_INVALID;
      add_edge(keys, b, v, t - 1);
    }
  }
  return csr_from_edges(keys, n, id_bytes, out);
}

// Sorted edge file (ReadSortedEdgeFile, graph_io.h:385-670, records parsed as
// in connect_io.h:216-260): '%' comment lines, a header "<type> n m", then
// records "e u w" of 1-based endpoints, one per undirected edge; other
// records are skipped.
int cc_read_edge_list(const char *path, uint32_t id_bytes, cc_host_graph *out) {
  if (!out || (id_bytes != 4 && id_bytes != 8)) return CC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::vector<char> buf;
  if (!slurp(path, buf)) return CC_ERR_INVALID;
  const char *p = buf.data(), *end = buf.data() + buf.size();
  uint64_t n = 0, m_hdr = 0;
  bool header = false;
  std::vector<uint64_t> keys;
  int b = 1;
  while (p < end) {
    const char *a = p, *e = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
    p = e + 1;
    while (a < e && (*a == ' ' || *a == '\t')) ++a;
    if (a >= e || *a == '%') continue;
    if (!header) {  // "<type> n m"
      while (a < e && *a != ' ' && *a != '\t') ++a;
      if (!next_uint(a, e, n) || !next_uint(a, e, m_hdr)) return CC_ERR_INVALID;
      if (n == 0 || n >= (1ull << 32)) return CC_ERR_INVALID;
      b = bits_for(n);
      keys.reserve(2 * m_hdr);
      header = true;
      continue;
    }
    if (*a != 'e') continue;
    ++a;
    uint64_t u, w;
    if (!next_uint(a, e, u) || !next_uint(a, e, w)) return CC_ERR_INVALID;
    if (u == 0 || w == 0 || u > n || w > n) return CC_ERR_INVALID;
    add_edge(keys, b, u - 1, w - 1);
  }
  if (!header) return CC_ERR_INVALID;
  return csr_from_edges(keys, n, id_bytes, out);
}

// Sorted binary edges (ReadSortedBinaryFile, graph_io.h:910-1175): uint64 n,
// uint64 m, then m pairs of uint64 1-based endpoints (host byte order).
int cc_read_binary_edges(const char *path, uint32_t id_bytes, cc_host_graph *out) {
  if (!out || (id_bytes != 4 && id_bytes != 8)) return CC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::vector<char> buf;
  if (!slurp(path, buf)) return CC_ERR_INVALID;
  const size_t len = buf.size() - 1;  // the appended newline
  if (len < 16) return CC_ERR_INVALID;
  uint64_t n = 0, m = 0;
  std::memcpy(&n, buf.data(), 8);
  std::memcpy(&m, buf.data() + 8, 8);
  if (n == 0 || n >= (1ull << 32) || m > (len - 16) / 16) return CC_ERR_INVALID;
  const int b = bits_for(n);
  std::vector<uint64_t> keys;
  keys.reserve(2 * m);
  for (uint64_t i = 0; i < m; ++i) {
    uint64_t uw[2];
    std::memcpy(uw, buf.data() + 16 + 16 * i, 16);
    if (uw[0] == 0 || uw[1] == 0 || uw[0] > n || uw[1] > n) return CC_ERR_INVALID;
    add_edge(keys, b, uw[0] - 1, uw[1] - 1);
  }
  return csr_from_edges(keys, n, id_bytes, out);
}

}  // extern "C"

/*
 * cc_oracle.c - CPU oracle for the connected-components hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the algorithms of
 * sebalamm/components that the GPU library replaces, so that tests/ can check
 * the GPU results and bench.py can time a CPU baseline.  The product never
 * links, loads or calls it.
 *
 * Parity pin: the reference ships no tests and no golden vectors; its only
 * fixture is example/simple.graph (components {1,2,3},{4,5,6}, canonical
 * labels [0,0,0,3,3,3]).  The reference itself cannot be compiled here (it
 * needs MPI, sparsehash, ips4o, tlx, boost, bliss/mxx and KaGen, which are
 * absent), so every restated solver is pinned to (a) that fixture and (b) an
 * independent union-find on the same inputs: connected components are unique,
 * so canonical labels (minimum vertex id per component) must agree exactly.
 *
 * Variates: the reference seeds std::default_random_engine per vertex and
 * draws std::exponential_distribution (exponential_contraction.h:469-472) or
 * mt19937 + uniform_int_distribution(0,99) (local_contraction.h:169-176).
 * Those streams only choose the contraction schedule; the oracle uses the
 * same counter-based variates as the GPU (SplitMix64 hash of seed, id, level
 * and an inverse-transform geometric sampler), restated here independently,
 * so that single stages can be compared bit for bit.
 *
 * Vertex ids are uint64 as in the reference (definitions.h:47-48); pair keys
 * need n < 2^32.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint64_t u64;
typedef uint32_t u32;

#define OR_NONE (~(u64)0)

/* ---------------------------------------------------------------- helpers */

static u64 mix64(u64 z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

u64 or_hash3(u64 seed, u64 a, u64 b) {
  return mix64(mix64(mix64(seed) ^ a) ^ (b * 0xd6e8feb86659fd93ull));
}

/* exp(x), x <= 0: reduction by ln 2 and a 30-term Taylor series in a fixed
   order (built with -ffp-contract=off), identical on every IEEE host. */
static double det_exp(double x) {
  const double ln2 = 0.6931471805599453094172321;
  double kf = floor(x / ln2 + 0.5);
  volatile double r = x - kf * ln2;
  double rr = r, term = 1.0, sum = 1.0;
  for (int i = 1; i < 30; ++i) {
    term = term * rr;
    term = term / (double)i;
    sum = sum + term;
  }
  return ldexp(sum, (int)kf);
}

/* T[k-1] = floor(2^64 exp(-beta k)), k = 1..len (len <= 4096). */
int or_geo_table(double beta, u64 *out, int cap) {
  int len = 0;
  if (!(beta > 0.0)) return 0;
  for (int k = 1; k <= 4096; ++k) {
    double x = ldexp(det_exp(-beta * (double)k), 64);
    if (x < 1.0) break;
    u64 v = x >= 18446744073709551615.0 ? ~(u64)0 : (u64)x;
    if (out && len < cap) out[len] = v;
    ++len;
  }
  return len;
}

/* floor(Exp(beta)) from a uniform word u: #{k : u < T[k-1]}. */
static u64 geo_dev(u64 u, const u64 *T, int len) {
  u64 d = 0;
  while ((int)d < len && u < T[d]) ++d;
  return d;
}

/* LSD radix sort of u64 keys, 16-bit digits, only the passes `bits` needs. */
static void radix_u64(u64 *a, u64 n, int bits) {
  if (n < 2) return;
  u64 *tmp = (u64 *)malloc(sizeof(u64) * n);
  u64 *cnt = (u64 *)malloc(sizeof(u64) * 65536);
  u64 *src = a, *dst = tmp;
  for (int sh = 0; sh < bits; sh += 16) {
    memset(cnt, 0, sizeof(u64) * 65536);
    for (u64 i = 0; i < n; ++i) cnt[(src[i] >> sh) & 0xffff]++;
    u64 run = 0;
    for (int d = 0; d < 65536; ++d) {
      u64 t = cnt[d];
      cnt[d] = run;
      run += t;
    }
    for (u64 i = 0; i < n; ++i) dst[cnt[(src[i] >> sh) & 0xffff]++] = src[i];
    u64 *t = src;
    src = dst;
    dst = t;
  }
  if (src != a) memcpy(a, src, sizeof(u64) * n);
  free(tmp);
  free(cnt);
}

static int bits_for(u64 x) {
  int b = 1;
  while (b < 64 && ((u64)1 << b) < x) ++b;
  return b;
}

/* Contiguous split of n vertices over P ranks: n/P + (r < n%P)
   (graph_io.h:308-313). */
static u64 rank_of(u64 v, u64 n, u64 P) {
  u64 q = n / P, rm = n % P, big = rm * (q + 1);
  return v < big ? v / (q + 1) : rm + (q ? (v - big) / q : 0);
}
static u64 rank_begin(u64 r, u64 n, u64 P) {
  u64 q = n / P, rm = n % P;
  return r < rm ? r * (q + 1) : rm * (q + 1) + (r - rm) * q;
}

/* --------------------------------------------------- second oracle: union-find
   Own code, 64-bit safe (the reference's UnionFind truncates to int,
   union_find.h:41-42).  Union by smaller id, so roots are component minima. */
static u64 uf_root(u64 *p, u64 v) {
  u64 r = v;
  while (p[r] != r) r = p[r];
  while (p[v] != r) {
    u64 nx = p[v];
    p[v] = r;
    v = nx;
  }
  return r;
}

int or_uf_labels(u64 n, const u64 *rp, const u64 *col, u64 *out) {
  for (u64 v = 0; v < n; ++v) out[v] = v;
  for (u64 v = 0; v < n; ++v)
    for (u64 e = rp[v]; e < rp[v + 1]; ++e) {
      u64 a = uf_root(out, v), b = uf_root(out, col[e]);
      if (a == b) continue;
      if (a < b) out[b] = a;
      else out[a] = b;
    }
  for (u64 v = 0; v < n; ++v) out[v] = uf_root(out, v);
  return 0;
}

/* lab[v] <- min vertex id with the same label; labels must be < n. */
void or_canonicalize(u64 n, u64 *lab) {
  u64 *mn = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  for (u64 i = 0; i < n; ++i) mn[i] = OR_NONE;
  for (u64 v = 0; v < n; ++v)
    if (v < mn[lab[v]]) mn[lab[v]] = v;
  for (u64 v = 0; v < n; ++v) lab[v] = mn[lab[v]];
  free(mn);
}

typedef struct {
  u64 l, v;
} or_pair;

static int pair_cmp(const void *x, const void *y) {
  const or_pair *a = (const or_pair *)x, *b = (const or_pair *)y;
  if (a->l != b->l) return a->l < b->l ? -1 : 1;
  return a->v < b->v ? -1 : (a->v > b->v);
}

/* Labels that may exceed n (the reference's raw labels, e.g. n + gid):
   canonicalised through a sort of (label, vertex) pairs. */
void or_canonicalize_any(u64 n, u64 *lab) {
  or_pair *a = (or_pair *)malloc(sizeof(or_pair) * (n ? n : 1));
  for (u64 i = 0; i < n; ++i) {
    a[i].l = lab[i];
    a[i].v = i;
  }
  qsort(a, n, sizeof(or_pair), pair_cmp);
  for (u64 i = 0; i < n;) {
    u64 j = i, mn = a[i].v; /* sorted by (label, id): the first id is the minimum */
    while (j < n && a[j].l == a[i].l) ++j;
    for (u64 k = i; k < j; ++k) lab[a[k].v] = mn;
    i = j;
  }
  free(a);
}

/* ------------------------------------------------ BFS (utils.h:37-58)
   parent[w] = start for every w reached; the caller labels a vertex with the
   label of its BFS start.  Restricted to [lo, hi) when lo < hi (local
   vertices of one rank; ghosts carry no adjacency in a StaticGraph). */
static void bfs_range(u64 n, const u64 *rp, const u64 *col, u64 lo, u64 hi, u64 *parent,
                      unsigned char *marked, u64 *queue) {
  (void)n;
  for (u64 s = lo; s < hi; ++s) {
    if (marked[s]) continue;
    u64 qh = 0, qt = 0;
    queue[qt++] = s;
    marked[s] = 1;
    parent[s] = s;
    while (qh < qt) {
      u64 v = queue[qh++];
      for (u64 e = rp[v]; e < rp[v + 1]; ++e) {
        u64 w = col[e];
        if (w < lo || w >= hi) continue; /* ghost: no adjacency here */
        if (!marked[w]) {
          marked[w] = 1;
          parent[w] = s;
          queue[qt++] = w;
        }
      }
    }
  }
}

/* FindLocalComponents on P ranks (exponential_contraction.h:391-411):
   out[v] = gid of the BFS start of v's rank-local component = its minimum
   local id.  Ranks run in parallel (one thread per rank), as MPI ranks do. */
int or_local_components(u64 n, const u64 *rp, const u64 *col, u64 P, u64 *out) {
  unsigned char *marked = (unsigned char *)calloc(n ? n : 1, 1);
  u64 *queue = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  long long r;
#pragma omp parallel for schedule(dynamic, 1)
  for (r = 0; r < (long long)P; ++r) {
    u64 lo = rank_begin((u64)r, n, P), hi = rank_begin((u64)r + 1, n, P);
    if (lo < hi) bfs_range(n, rp, col, lo, hi, out, marked, queue + lo);
  }
  free(marked);
  free(queue);
  return 0;
}

/* ------------------------------------------------ quotient graph
   Graph over cluster ids: undirected edges {cl[v], cl[w]} with different
   ids, deduplicated, both directions.  New vertex ids are the clusters that
   own an edge, in increasing cluster order.  Output arrays are malloc'ed. */
typedef struct {
  u64 n, m;
  u64 *rp, *col, *vid; /* vid[new] = cluster id */
  u64 *newid;          /* per cluster id (< ncl): new id or OR_NONE */
} or_graph;

static void graph_free(or_graph *g) {
  free(g->rp);
  free(g->col);
  free(g->vid);
  free(g->newid);
  memset(g, 0, sizeof(*g));
}

static int n_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
static int thread_id(void) {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

static int keep_edge(u64 v, u64 w, const u64 *cl, int only_cut, u64 n, u64 P) {
  if (only_cut && rank_of(v, n, P) == rank_of(w, n, P)) return 0;
  return cl[v] != cl[w];
}

static void quotient(u64 n, const u64 *rp, const u64 *col, const u64 *cl, u64 ncl,
                     int only_cut, u64 P, or_graph *out) {
  int b = bits_for(ncl);
  u64 m = n ? rp[n] : 0, k = 0;
  u64 *keys = (u64 *)malloc(sizeof(u64) * (m ? m : 1));
  /* key emission in parallel, each thread over a contiguous vertex range (the
     ranks of the reference do this step concurrently) */
  int nt = n_threads(), used = 1;
  u64 *cnt = (u64 *)calloc((size_t)nt + 1, sizeof(u64));
#pragma omp parallel num_threads(nt)
  {
    int t = thread_id(), T = 1;
#ifdef _OPENMP
    T = omp_get_num_threads();
#endif
    u64 lo = n * (u64)t / (u64)T, hi = n * (u64)(t + 1) / (u64)T, c = 0;
    for (u64 v = lo; v < hi; ++v)
      for (u64 e = rp[v]; e < rp[v + 1]; ++e) c += keep_edge(v, col[e], cl, only_cut, n, P);
    cnt[t + 1] = c;
#pragma omp barrier
#pragma omp single
    {
      for (int i = 0; i < T; ++i) cnt[i + 1] += cnt[i];
      used = T;
    }
    u64 pos = cnt[t];
    for (u64 v = lo; v < hi; ++v)
      for (u64 e = rp[v]; e < rp[v + 1]; ++e)
        if (keep_edge(v, col[e], cl, only_cut, n, P)) keys[pos++] = (cl[v] << b) | cl[col[e]];
  }
  k = cnt[used];
  free(cnt);
  radix_u64(keys, k, 2 * b);
  u64 u = 0;
  for (u64 i = 0; i < k; ++i)
    if (i == 0 || keys[i] != keys[i - 1]) keys[u++] = keys[i];
  out->newid = (u64 *)malloc(sizeof(u64) * (ncl ? ncl : 1));
  for (u64 c = 0; c < ncl; ++c) out->newid[c] = OR_NONE;
  for (u64 i = 0; i < u; ++i) out->newid[keys[i] >> b] = 1;
  u64 nn = 0;
  for (u64 c = 0; c < ncl; ++c)
    if (out->newid[c] != OR_NONE) out->newid[c] = nn++;
  out->n = nn;
  out->m = u;
  out->rp = (u64 *)calloc(nn + 1, sizeof(u64));
  out->col = (u64 *)malloc(sizeof(u64) * (u ? u : 1));
  out->vid = (u64 *)malloc(sizeof(u64) * (nn ? nn : 1));
  const u64 mask = ((u64)1 << b) - 1;
  for (u64 i = 0; i < u; ++i) {
    out->rp[out->newid[keys[i] >> b] + 1]++;
    out->col[i] = out->newid[keys[i] & mask];
  }
  for (u64 i = 0; i < nn; ++i) out->rp[i + 1] += out->rp[i];
  for (u64 c = 0; c < ncl; ++c)
    if (out->newid[c] != OR_NONE) out->vid[out->newid[c]] = c;
  free(keys);
}

int or_contract(u64 n, const u64 *rp, const u64 *col, const u64 *cl, u64 ncl, u64 cut_parts,
                u64 *rp_out, u64 *col_out, u64 *vid_out, u64 *newid_out, u64 *n_out, u64 *m_out) {
  or_graph h;
  memset(&h, 0, sizeof(h));
  quotient(n, rp, col, cl, ncl, cut_parts > 0, cut_parts ? cut_parts : 1, &h);
  memcpy(rp_out, h.rp, sizeof(u64) * (h.n + 1));
  memcpy(col_out, h.col, sizeof(u64) * h.m);
  memcpy(vid_out, h.vid, sizeof(u64) * h.n);
  memcpy(newid_out, h.newid, sizeof(u64) * ncl);
  *n_out = h.n;
  *m_out = h.m;
  graph_free(&h);
  return 0;
}

/* ------------------------------------------- exponential-shift decomposition
   RunContractionLP (exponential_contraction.h:439-628) on a graph whose
   vertices are numbered in increasing label order: key = (dev << 32) | index,
   relax key[v] = min(key[v], key[w] + 2^32) (:527-549) until nothing changes.
   cluster[v] = index of the centre. */
int or_ldd(u64 n, const u64 *rp, const u64 *col, const u64 *vid, u64 seed, u64 level, double beta,
           u64 *cluster) {
  u64 T[4096];
  int len = or_geo_table(beta, T, 4096);
  u64 *key = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  for (u64 v = 0; v < n; ++v) key[v] = (geo_dev(or_hash3(seed, vid[v], level), T, len) << 32) | v;
  int rounds = 0, changed = 1;
  while (changed) {
    changed = 0;
    ++rounds;
    for (u64 v = 0; v < n; ++v) {
      u64 best = key[v];
      for (u64 e = rp[v]; e < rp[v + 1]; ++e) {
        u64 kw = key[col[e]] + ((u64)1 << 32);
        if (kw < best) best = kw;
      }
      if (best < key[v]) {
        key[v] = best;
        changed = 1;
      }
    }
  }
  for (u64 v = 0; v < n; ++v) cluster[v] = key[v] & 0xffffffffull;
  free(key);
  return rounds;
}

/* Local contraction sweeps (local_contraction.h:166-255): uniform deviate in
   [0, 99], key = (dev << 32) | index, two Jacobi sweeps of the minimum over
   the closed neighbourhood; cluster = low word. */
int or_local_sweeps(u64 n, const u64 *rp, const u64 *col, const u64 *vid, u64 seed, u64 level,
                    u64 *cluster) {
  u64 *k0 = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  u64 *k1 = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  for (u64 v = 0; v < n; ++v) {
    u64 d = ((or_hash3(seed, vid[v], level) >> 32) * 100ull) >> 32;
    k0[v] = (d << 32) | v;
  }
  for (int sweep = 0; sweep < 2; ++sweep) {
    u64 *in = sweep ? k1 : k0, *outk = sweep ? k0 : k1;
    for (u64 v = 0; v < n; ++v) {
      u64 best = in[v];
      for (u64 e = rp[v]; e < rp[v + 1]; ++e)
        if (in[col[e]] < best) best = in[col[e]];
      outk[v] = best;
    }
  }
  for (u64 v = 0; v < n; ++v) cluster[v] = k0[v] & 0xffffffffull;
  free(k0);
  free(k1);
  return 0;
}

/* ---------------------------------------------- sequential base case
   AllReduce::FindComponents (all_reduce.h:46-250): gather vertices in rank
   order, BFS on the gathered graph, label = label of the first gathered vertex
   of the component (FindLocalComponents :141-158).  Vertices are gathered in
   increasing id here. */
int or_allreduce(u64 n, const u64 *rp, const u64 *col, const u64 *lab_in, u64 *lab_out) {
  unsigned char *marked = (unsigned char *)calloc(n ? n : 1, 1);
  u64 *parent = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  u64 *queue = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  bfs_range(n, rp, col, 0, n, parent, marked, queue);
  for (u64 v = 0; v < n; ++v) lab_out[v] = lab_in[parent[v]];
  free(marked);
  free(parent);
  free(queue);
  return 0;
}

/* level recursion shared by the exponential and the local contraction.
   Graph g (vertex index order = label order), vid = labels (gids); writes
   the final label of every vertex into out. */
typedef struct {
  double beta;
  u64 seed, limit;
  int local; /* 0: exponential shifts (edge limit), 1: local sweeps (vertex limit) */
  int levels, max_levels;
  u64 rounds_total;
} or_rec;

static void levels(or_rec *R, u64 n, const u64 *rp, const u64 *col, const u64 *vid, u64 level,
                   u64 *out) {
  if (n == 0) return;
  u64 m = rp[n];
  if ((int)level > R->levels) R->levels = (int)level;
  int base = R->local ? (n <= R->limit || m == 0) : (m <= R->limit);
  if (base || (int)level >= R->max_levels) {
    or_allreduce(n, rp, col, vid, out); /* RunSequentialCC */
    return;
  }
  u64 *cl = (u64 *)malloc(sizeof(u64) * n);
  if (R->local) or_local_sweeps(n, rp, col, vid, R->seed, level, cl);
  else R->rounds_total += (u64)or_ldd(n, rp, col, vid, R->seed, level, R->beta, cl);
  or_graph h;
  memset(&h, 0, sizeof(h));
  quotient(n, rp, col, cl, n, 0, 1, &h);
  u64 *vid2 = (u64 *)malloc(sizeof(u64) * (h.n ? h.n : 1));
  for (u64 i = 0; i < h.n; ++i) vid2[i] = vid[h.vid[i]];
  u64 *sub = (u64 *)malloc(sizeof(u64) * (h.n ? h.n : 1));
  levels(R, h.n, h.rp, h.col, vid2, level + 1, sub);
  /* UndoContraction (dynamic_contraction.h:568-658): every vertex takes the
     final label of its centre; centres without edges keep their own label */
  for (u64 v = 0; v < n; ++v) {
    u64 c = cl[v], id = h.newid[c];
    out[v] = id != OR_NONE ? sub[id] : vid[c];
  }
  free(sub);
  free(vid2);
  free(cl);
  graph_free(&h);
}

/* ExponentialContraction::FindComponents, default path
   (exponential_contraction.h:59-64, 217-305):
     FindLocalComponents -> local contraction (cag_builder.h:160-230):
       cv(v) = v if v is an interface vertex (has a neighbour on another rank)
               else its local component label;
       lcag = quotient graph under cv (vertices without edges stay inactive)
     PerformDecomposition (:364-389) with sequential_limit = (m/P)*seq
     (ComputeSequentialLimit :1287-1292), UndoContraction, then
     ApplyToLocalComponents (:876-889): label(v) = lcag label of cv(v).
   raw_out gets these (non-canonical) labels.  Returns the number of levels. */
int or_exp_contraction(u64 n, const u64 *rp, const u64 *col, u64 P, double beta, u64 seq,
                       int fixed_seq, u64 seed, u64 *raw_out, u64 *rounds_out) {
  if (n == 0) return 0;
  u64 m = rp[n];
  u64 *lab = (u64 *)malloc(sizeof(u64) * n);
  or_local_components(n, rp, col, P, lab);
  u64 *cv = (u64 *)malloc(sizeof(u64) * n);
  long long vv;
#pragma omp parallel for schedule(static)
  for (vv = 0; vv < (long long)n; ++vv) {
    u64 v = (u64)vv;
    int iface = 0;
    u64 r = rank_of(v, n, P);
    for (u64 e = rp[v]; e < rp[v + 1] && !iface; ++e) iface = rank_of(col[e], n, P) != r;
    cv[v] = iface ? v : lab[v];
  }
  or_graph h;
  memset(&h, 0, sizeof(h));
  quotient(n, rp, col, cv, n, 0, 1, &h);
  or_rec R;
  memset(&R, 0, sizeof(R));
  R.beta = beta;
  R.seed = seed;
  R.limit = fixed_seq ? seq : (m / P) * seq;
  R.max_levels = 63;
  u64 *sub = (u64 *)malloc(sizeof(u64) * (h.n ? h.n : 1));
  /* lcag labels are gids; its vertex order is gid order */
  levels(&R, h.n, h.rp, h.col, h.vid, 1, sub);
#pragma omp parallel for schedule(static)
  for (vv = 0; vv < (long long)n; ++vv) {
    u64 id = h.newid[cv[vv]];
    raw_out[vv] = id != OR_NONE ? sub[id] : cv[vv];
  }
  if (rounds_out) *rounds_out = R.rounds_total;
  free(sub);
  free(cv);
  free(lab);
  graph_free(&h);
  return R.levels;
}

/* LocalContraction::FindComponents on a DynamicGraphCommunicator
   (local_contraction.h:78-86, 157-348): sweeps + contraction per level until
   at most `seq` vertices remain (an absolute count, :119), then the
   sequential base case, then UndoContraction. */
int or_local_contraction(u64 n, const u64 *rp, const u64 *col, u64 seq, u64 seed, u64 *out) {
  if (n == 0) return 0;
  u64 *vid = (u64 *)malloc(sizeof(u64) * n);
  for (u64 v = 0; v < n; ++v) vid[v] = v;
  or_rec R;
  memset(&R, 0, sizeof(R));
  R.seed = seed;
  R.limit = seq;
  R.local = 1;
  R.max_levels = 63;
  levels(&R, n, rp, col, vid, 1, out);
  free(vid);
  return R.levels;
}

/* Propagation (propagation.h:72-149): in-place minimum over the neighbours
   until no label changes.  Returns the number of rounds. */
int or_labels(u64 n, const u64 *rp, const u64 *col, u64 *lab) {
  int rounds = 0, changed = 1;
  for (u64 v = 0; v < n; ++v) lab[v] = v;
  while (changed) {
    changed = 0;
    ++rounds;
    for (u64 v = 0; v < n; ++v) {
      u64 l = lab[v];
      for (u64 e = rp[v]; e < rp[v + 1]; ++e)
        if (lab[col[e]] < l) l = lab[col[e]];
      if (l < lab[v]) {
        lab[v] = l;
        changed = 1;
      }
    }
  }
  return rounds;
}

/* ShortcutPropagation (shortcut_propagation.h:124-376), one rank, Jacobi
   rounds on f (the graph labels) and nf (labels_):
     FindMinLabels: nf[v] = min over N[v] of f
     Shortcut: updates (f[v] -> nf[v]) for every v whose label drops, requests
       f[nf[v]] (only for heavy-hitter labels when hitters > 0); every answer
       for target t lowers nf[u] of all u with nf[u] == t
     CheckConvergence: stop when nf == f; PropagateLabels: f = nf.
   lab holds the initial labels and receives the final ones.  Returns rounds. */
int or_shortcut(u64 n, const u64 *rp, const u64 *col, u64 *lab, u64 hitters) {
  u64 *nf = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  u64 *upd = (u64 *)malloc(sizeof(u64) * (n ? n : 1));
  unsigned char *heavy = (unsigned char *)calloc(n ? n : 1, 1);
  u64 *cnt = hitters ? (u64 *)malloc(sizeof(u64) * (n ? n : 1)) : NULL;
  int rounds = 0;
  for (;;) {
    ++rounds;
    for (u64 v = 0; v < n; ++v) upd[v] = OR_NONE;
    for (u64 v = 0; v < n; ++v) {
      u64 best = lab[v];
      for (u64 e = rp[v]; e < rp[v + 1]; ++e)
        if (lab[col[e]] < best) best = lab[col[e]];
      nf[v] = best;
      if (best < lab[v] && best < upd[lab[v]]) upd[lab[v]] = best;
    }
    if (hitters) {
      for (u64 v = 0; v < n; ++v) cnt[v] = 0;
      for (u64 v = 0; v < n; ++v) cnt[nf[v]]++;
      for (u64 v = 0; v < n; ++v)
        if (cnt[v] > n / hitters) heavy[v] = 1;
    }
    int changed = 0;
    for (u64 u = 0; u < n; ++u) {
      u64 t = nf[u], r = t;
      if (!hitters || heavy[t])
        if (lab[t] < r) r = lab[t];
      if (upd[t] < r) r = upd[t];
      nf[u] = r;
      if (r != lab[u]) changed = 1;
    }
    for (u64 u = 0; u < n; ++u) lab[u] = nf[u];
    if (!changed) break;
  }
  free(nf);
  free(upd);
  free(heavy);
  free(cnt);
  return rounds;
}

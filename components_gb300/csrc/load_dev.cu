// load_dev.cu - the reference's input files read straight into a device CSR.
//
// The drivers read their input with GraphIO (lib/io/graph_io.h): METIS text
// (ReadMETISFile, :281-382) and the sorted binary edge file
// (ReadSortedBinaryFile, :910-1175).  The host readers of csrc/gen.cpp parse
// them on one host thread and build the CSR in host memory, which then
// crosses the host link.  Here the file's bytes go to the device once (read
// into the context's page-locked staging, one copy) and everything else runs
// there: the newline positions and the number tokens of a METIS file are
// found by parallel scans over the bytes, every token becomes the two
// directed keys of its edge, and one radix sort, an adjacent-unique pass and
// a binary search per vertex give the CSR with sorted rows.  The result is
// the host reader's CSR bit for bit: the same comment, header and token rules
// (a line whose first character is '%' is a comment; the first other line is
// the header "n m ..."; then one line per vertex, whose tokens are the
// unsigned decimals before the first character that is neither a digit nor a
// space, tab or carriage return; missing trailing lines are isolated
// vertices), self-loops and repeated edges dropped.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/cc_gpu.h"
#include "ctx.h"
#include "scan.cuh"

namespace ccg {
namespace {

constexpr uint32_t kNoVertex = 0xffffffffu;

__device__ __forceinline__ bool is_digit(uint8_t c) { return c >= '0' && c <= '9'; }
__device__ __forceinline__ bool is_blank(uint8_t c) { return c == ' ' || c == '\t' || c == '\r'; }

// Scan functors: newline flags and their positions; token starts and theirs.
struct GetNewline {
  const uint8_t *b;
  __device__ uint32_t operator()(uint64_t i) const { return b[i] == '\n'; }
};
struct GetTokenStart {
  const uint8_t *b;
  __device__ uint32_t operator()(uint64_t i) const {
    return is_digit(b[i]) && (i == 0 || !is_digit(b[i - 1]));
  }
};
struct PutNothing {  // a counting pass
  __device__ void operator()(uint64_t, uint32_t, uint32_t) const {}
};
struct PutPosition {
  uint32_t *pos;
  __device__ void operator()(uint64_t i, uint32_t excl, uint32_t f) const {
    if (f) pos[excl] = (uint32_t)i;
  }
};
// Lines that are not comments, and their ranks among those.
struct GetNotComment {
  const uint8_t *b;
  const uint32_t *nl;
  __device__ uint32_t operator()(uint64_t k) const {
    const uint32_t start = k ? nl[k - 1] + 1 : 0u;
    return b[start] != '%';  // an empty line starts at its own newline: not a comment
  }
};
struct PutVertex {
  const uint8_t *b;
  const uint32_t *nl;
  uint64_t n;
  uint32_t *vtx;  // per line: its vertex, or kNoVertex (comment, header, beyond n)
  __device__ void operator()(uint64_t k, uint32_t excl, uint32_t f) const {
    vtx[k] = (f && excl >= 1 && excl <= n) ? excl - 1 : kNoVertex;
  }
};

// Line of byte position p: the first newline at or after p (binary search).
__device__ __forceinline__ uint32_t line_of(const uint32_t *__restrict__ nl, uint32_t lines,
                                            uint32_t p) {
  uint32_t lo = 0, hi = lines;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (nl[mid] < p) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// bad[k] = the first position of line k holding a character that ends its
// tokens (not a digit, blank or newline); lines without one keep their
// newline position.
__global__ void k_first_bad(const uint8_t *__restrict__ b, uint64_t len, const uint32_t *__restrict__ nl,
                            uint32_t lines, uint32_t *__restrict__ bad) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t c = b[i];
    if (is_digit(c) || is_blank(c) || c == '\n') continue;
    atomicMin(bad + line_of(nl, lines, (uint32_t)i), (uint32_t)i);
  }
}

// Every token of a vertex line becomes the two directed keys of its edge
// ((v << bits) | u and the reverse); tokens that do not count, and
// self-loops, become the marker ~0 (sorted after every key).  An id outside
// [1, n] sets the error word.
__global__ void k_metis_keys(const uint8_t *__restrict__ b, const uint32_t *__restrict__ tok,
                             uint64_t ntok, const uint32_t *__restrict__ nl, uint32_t lines,
                             const uint32_t *__restrict__ vtx, const uint32_t *__restrict__ bad,
                             uint64_t n, int bits, uint64_t *__restrict__ keys, int *err) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ntok;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = tok[i];
    const uint32_t k = line_of(nl, lines, p);
    uint64_t a = ~0ull, r = ~0ull;
    const uint32_t v = vtx[k];
    if (v != kNoVertex && p < bad[k]) {
      uint64_t t = 0;  // as the host reader: no overflow check, the range test below decides
      for (uint32_t q = p; is_digit(b[q]); ++q) t = 10 * t + (uint64_t)(b[q] - '0');
      if (t == 0 || t > n) {
        set_err(err, kErrBadId);
      } else if (t - 1 != v) {
        a = ((uint64_t)v << bits) | (t - 1);
        r = ((t - 1) << bits) | v;
      }
    }
    keys[2 * i] = a;
    keys[2 * i + 1] = r;
  }
}

// The binary file's m pairs of 1-based uint64 endpoints, as keys.
__global__ void k_binary_keys(const uint64_t *__restrict__ pairs, uint64_t m, uint64_t n, int bits,
                              uint64_t *__restrict__ keys, int *err) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t u = pairs[2 * i], w = pairs[2 * i + 1];
    uint64_t a = ~0ull, r = ~0ull;
    if (u == 0 || w == 0 || u > n || w > n) {
      set_err(err, kErrBadId);
    } else if (u != w) {
      a = ((u - 1) << bits) | (w - 1);
      r = ((w - 1) << bits) | (u - 1);
    }
    keys[2 * i] = a;
    keys[2 * i + 1] = r;
  }
}

// rp[v] = the first key with source >= v (v in [0, n]); col = the targets.
template <class T>
__global__ void k_keys_csr(const uint64_t *__restrict__ keys, uint64_t nk, uint64_t n, int bits,
                           uint64_t *__restrict__ rp, T *__restrict__ col) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (uint64_t v = t; v <= n; v += stride) {
    uint64_t lo = 0, hi = nk;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if ((keys[mid] >> bits) < v) lo = mid + 1;
      else hi = mid;
    }
    rp[v] = lo;
  }
  const uint64_t mask = (1ull << bits) - 1;
  for (uint64_t e = t; e < nk; e += stride) col[e] = (T)(keys[e] & mask);
}

int bits_of_n(uint64_t x) {
  int b = 1;
  while (b < 64 && (1ull << b) < x) ++b;
  return b;
}

}  // namespace
}  // namespace ccg

using ccg::DevBuf;
using ccg::Error;

namespace {

// The whole file plus one '\n' (every line then ends with a newline) in the
// context's page-locked staging buffer; *len counts the appended newline.
uint8_t *read_pinned(cc_ctx *C, const char *path, uint64_t *len) {
  FILE *f = path ? std::fopen(path, "rb") : nullptr;
  if (!f) throw Error(CC_ERR_INVALID, "cannot open the input file");
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    std::fclose(f);
    throw Error(CC_ERR_INVALID, "cannot size the input file");
  }
  if (!C->stager) C->stager.reset(new ccg::HostStager());
  uint8_t *buf = C->stager->staging((size_t)sz + 16);
  if (!buf) {
    std::fclose(f);
    throw Error(CC_ERR_OOM, "no page-locked staging for the input file");
  }
  const size_t got = sz ? std::fread(buf, 1, (size_t)sz, f) : 0;
  std::fclose(f);
  if (got != (size_t)sz) throw Error(CC_ERR_INVALID, "short read of the input file");
  buf[sz] = '\n';
  *len = (uint64_t)sz + 1;
  return buf;
}

// Unsigned decimal at p (spaces, tabs and carriage returns skipped first), as
// the host reader; false when the line has none there.
bool next_uint_h(const uint8_t *&p, const uint8_t *eol, uint64_t &v) {
  while (p < eol && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
  if (p >= eol || *p < '0' || *p > '9') return false;
  v = 0;
  while (p < eol && *p >= '0' && *p <= '9') v = 10 * v + (uint64_t)(*p++ - '0');
  return true;
}

// The host readers' vertex-count rule.
void check_ids(uint64_t n, uint32_t id_bytes) {
  if (n == 0 || n >= (1ull << 32) || (id_bytes == 4 && n >= 0xffffffffull))
    throw Error(CC_ERR_INVALID, "vertex count out of range");
}

// The first bytes of the file (up to cap) plus the file size, for a size
// query that needs only the header.
std::vector<uint8_t> read_head(const char *path, uint64_t cap, uint64_t *size) {
  FILE *f = path ? std::fopen(path, "rb") : nullptr;
  if (!f) throw Error(CC_ERR_INVALID, "cannot open the input file");
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    std::fclose(f);
    throw Error(CC_ERR_INVALID, "cannot size the input file");
  }
  std::vector<uint8_t> buf((size_t)std::min<uint64_t>((uint64_t)sz, cap) + 1);
  const size_t got = std::fread(buf.data(), 1, buf.size() - 1, f);
  std::fclose(f);
  if (got != buf.size() - 1) throw Error(CC_ERR_INVALID, "short read of the input file");
  buf.back() = '\n';
  *size = (uint64_t)sz;
  return buf;
}

// The METIS header: the first line that is not a comment.  false when the
// buffer ends before one.
bool metis_header(const uint8_t *hb, uint64_t len, uint64_t *n, uint64_t *m_hdr) {
  const uint8_t *p = hb, *end = hb + len, *a = nullptr, *e = nullptr;
  while (p < end) {
    a = p;
    e = static_cast<const uint8_t *>(std::memchr(p, '\n', (size_t)(end - p)));
    p = e + 1;
    if (*a != '%') break;
    a = nullptr;
  }
  if (!a) return false;
  if (!next_uint_h(a, e, *n) || !next_uint_h(a, e, *m_hdr)) throw Error(CC_ERR_INVALID, "no METIS header");
  return true;
}

// Sorted, deduplicated keys (marker ~0 dropped) into the caller's CSR.
void keys_to_csr(cc_ctx *C, uint64_t *keys, uint64_t nk, uint64_t n, int bits, uint32_t id_bytes,
                 uint64_t *row_ptr, void *col, uint64_t cap, uint64_t *m_dir, ccg::Counters &c) {
  cudaStream_t s = C->stream;
  DevBuf tmp(8 * (nk ? nk : 1), s, C->pool), uniq(8 * (nk ? nk : 1), s, C->pool), cnt(4, s, C->pool);
  uint64_t u = 0;
  const uint64_t *sorted = keys;
  if (nk) {
    sorted = ccg::radix_sort_u64(keys, tmp.as<uint64_t>(), nk, 2 * bits, s, C->pool, c);
    ccg::unique_sorted_keys(sorted, nk, uniq.as<uint64_t>(), cnt.as<uint32_t>(), s, C->pool, c);
    uint32_t nu = 0;
    uint64_t last = 0;
    CCG_CUDA(cudaMemcpyAsync(&nu, cnt.p, 4, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    if (nu) {
      CCG_CUDA(cudaMemcpyAsync(&last, uniq.as<uint64_t>() + nu - 1, 8, cudaMemcpyDeviceToHost, s));
      CCG_CUDA(cudaStreamSynchronize(s));
    }
    u = nu - (nu && last == ~0ull ? 1 : 0);  // the marker sorts last
  }
  ccg::throw_on_kernel_error(C, s);  // ids outside [1, n]
  *m_dir = u;
  if (u > cap) throw Error(CC_ERR_INVALID, "col capacity below the entries read");
  const unsigned grid = ccg::grid_for(std::max<uint64_t>(n + 1, u), ccg::kBlock, ccg::num_sms() * 16);
  if (id_bytes == 8)
    ccg::k_keys_csr<uint64_t><<<grid, ccg::kBlock, 0, s>>>(uniq.as<uint64_t>(), u, n, bits, row_ptr,
                                                          static_cast<uint64_t *>(col));
  else
    ccg::k_keys_csr<uint32_t><<<grid, ccg::kBlock, 0, s>>>(uniq.as<uint64_t>(), u, n, bits, row_ptr,
                                                          static_cast<uint32_t *>(col));
  CCG_LAUNCH_CHECK();
  CCG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

extern "C" {

int cc_read_metis_device(cc_ctx *ctx, const char *path, uint32_t id_bytes, uint64_t *row_ptr,
                         void *col, uint64_t cap, uint64_t *n_out, uint64_t *m_dir) {
  return ccg::guard([&] {
    if ((id_bytes != 4 && id_bytes != 8) || !n_out || !m_dir || (row_ptr && cap && !col))
      throw Error(CC_ERR_INVALID, "bad METIS loader arguments");
    uint64_t n = 0, m_hdr = 0;
    if (!row_ptr) {  // size query: the header, and every entry needs a token of two bytes or more
      uint64_t size = 0;
      std::vector<uint8_t> head = read_head(path, 1 << 20, &size);
      if (!metis_header(head.data(), head.size(), &n, &m_hdr)) {
        head = read_head(path, ~0ull, &size);
        if (!metis_header(head.data(), head.size(), &n, &m_hdr)) throw Error(CC_ERR_INVALID, "no METIS header");
      }
      check_ids(n, id_bytes);
      *n_out = n;
      *m_dir = size + 1;
      return;
    }
    cc_ctx *C = ctx ? ctx : ccg::default_context();
    CCG_CUDA(cudaSetDevice(C->device));
    uint64_t len = 0;
    const uint8_t *hb = read_pinned(C, path, &len);
    if (len >= 0xffffffffull) throw Error(CC_ERR_UNSUPPORTED, "a METIS file of 4 GB or more");
    if (!metis_header(hb, len, &n, &m_hdr)) throw Error(CC_ERR_INVALID, "no METIS header");
    check_ids(n, id_bytes);
    *n_out = n;
    cudaStream_t s = C->stream;
    ccg::Counters c;
    CCG_CUDA(cudaMemsetAsync(C->d_err, 0, sizeof(int), s));
    DevBuf db(len, s, C->pool), cnt(8, s, C->pool);
    CCG_CUDA(cudaMemcpyAsync(db.p, hb, len, cudaMemcpyHostToDevice, s));
    const uint8_t *b = db.as<uint8_t>();
    uint32_t *d_cnt = cnt.as<uint32_t>();
    uint32_t h_cnt[2] = {0, 0};
    // newline positions
    ccg::scan_generic(len, ccg::GetNewline{b}, ccg::PutNothing{}, d_cnt, s, C->pool, c);
    CCG_CUDA(cudaMemcpyAsync(h_cnt, d_cnt, 4, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    const uint32_t lines = h_cnt[0];
    DevBuf nl(4 * (uint64_t)lines, s, C->pool), vtx(4 * (uint64_t)lines, s, C->pool),
        bad(4 * (uint64_t)lines, s, C->pool);
    ccg::scan_generic(len, ccg::GetNewline{b}, ccg::PutPosition{nl.as<uint32_t>()}, nullptr, s, C->pool, c);
    // lines that are not comments: the first is the header, the next n the vertices
    ccg::scan_generic(lines, ccg::GetNotComment{b, nl.as<uint32_t>()},
                      ccg::PutVertex{b, nl.as<uint32_t>(), n, vtx.as<uint32_t>()}, nullptr, s, C->pool, c);
    CCG_CUDA(cudaMemcpyAsync(bad.p, nl.p, 4 * (uint64_t)lines, cudaMemcpyDeviceToDevice, s));
    const unsigned grid = ccg::grid_for(len, ccg::kBlock, ccg::num_sms() * 16);
    ccg::k_first_bad<<<grid, ccg::kBlock, 0, s>>>(b, len, nl.as<uint32_t>(), lines, bad.as<uint32_t>());
    CCG_LAUNCH_CHECK();
    // token positions
    ccg::scan_generic(len, ccg::GetTokenStart{b}, ccg::PutNothing{}, d_cnt + 1, s, C->pool, c);
    CCG_CUDA(cudaMemcpyAsync(h_cnt + 1, d_cnt + 1, 4, cudaMemcpyDeviceToHost, s));
    CCG_CUDA(cudaStreamSynchronize(s));
    const uint64_t ntok = h_cnt[1];
    if (2 * ntok >= (1ull << 32)) throw Error(CC_ERR_UNSUPPORTED, "2^31 tokens or more");
    DevBuf tok(4 * (ntok ? ntok : 1), s, C->pool), keys(16 * (ntok ? ntok : 1), s, C->pool);
    ccg::scan_generic(len, ccg::GetTokenStart{b}, ccg::PutPosition{tok.as<uint32_t>()}, nullptr, s,
                      C->pool, c);
    const int bits = ccg::bits_of_n(n);
    if (ntok) {
      ccg::k_metis_keys<<<ccg::grid_for(ntok, ccg::kBlock, ccg::num_sms() * 16), ccg::kBlock, 0, s>>>(
          b, tok.as<uint32_t>(), ntok, nl.as<uint32_t>(), lines, vtx.as<uint32_t>(), bad.as<uint32_t>(),
          n, bits, keys.as<uint64_t>(), C->d_err);
      CCG_LAUNCH_CHECK();
    }
    keys_to_csr(C, keys.as<uint64_t>(), 2 * ntok, n, bits, id_bytes, row_ptr, col, cap, m_dir, c);
  });
}

int cc_read_binary_edges_device(cc_ctx *ctx, const char *path, uint32_t id_bytes, uint64_t *row_ptr,
                                void *col, uint64_t cap, uint64_t *n_out, uint64_t *m_dir) {
  return ccg::guard([&] {
    if ((id_bytes != 4 && id_bytes != 8) || !n_out || !m_dir || (row_ptr && cap && !col))
      throw Error(CC_ERR_INVALID, "bad binary loader arguments");
    auto header = [&](const uint8_t *hb, uint64_t bytes, uint64_t *n, uint64_t *m) {
      if (bytes < 16) throw Error(CC_ERR_INVALID, "binary file shorter than its header");
      std::memcpy(n, hb, 8);
      std::memcpy(m, hb + 8, 8);
      if (*m > (bytes - 16) / 16) throw Error(CC_ERR_INVALID, "binary file shorter than its m pairs");
      check_ids(*n, id_bytes);
      if (2 * *m >= (1ull << 32)) throw Error(CC_ERR_UNSUPPORTED, "2^31 pairs or more");
    };
    uint64_t n = 0, m = 0;
    if (!row_ptr) {  // size query
      uint64_t size = 0;
      std::vector<uint8_t> head = read_head(path, 16, &size);
      header(head.data(), size, &n, &m);
      *n_out = n;
      *m_dir = 2 * m;
      return;
    }
    cc_ctx *C = ctx ? ctx : ccg::default_context();
    CCG_CUDA(cudaSetDevice(C->device));
    uint64_t len = 0;
    const uint8_t *hb = read_pinned(C, path, &len);
    header(hb, len - 1, &n, &m);  // without the appended newline
    *n_out = n;
    cudaStream_t s = C->stream;
    ccg::Counters c;
    CCG_CUDA(cudaMemsetAsync(C->d_err, 0, sizeof(int), s));
    DevBuf pairs(16 * (m ? m : 1), s, C->pool), keys(16 * (m ? m : 1), s, C->pool);
    if (m) CCG_CUDA(cudaMemcpyAsync(pairs.p, hb + 16, 16 * m, cudaMemcpyHostToDevice, s));
    const int bits = ccg::bits_of_n(n);
    if (m) {
      ccg::k_binary_keys<<<ccg::grid_for(m, ccg::kBlock, ccg::num_sms() * 16), ccg::kBlock, 0, s>>>(
          pairs.as<uint64_t>(), m, n, bits, keys.as<uint64_t>(), C->d_err);
      CCG_LAUNCH_CHECK();
    }
    keys_to_csr(C, keys.as<uint64_t>(), 2 * m, n, bits, id_bytes, row_ptr, col, cap, m_dir, c);
  });
}

}  // extern "C"

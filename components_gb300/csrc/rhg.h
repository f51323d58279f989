// rhg.h - the random hyperbolic graph (threshold model) as pure functions of
// (seed, vertex index), evaluated bit-identically by the host generator
// (gen.cpp, g++) and the device generator (gen_dev.cu, nvcc).
//
// Model (Krioukov et al., "Hyperbolic geometry of complex networks", Phys.
// Rev. E 82, 2010; the rhg generator the reference drivers call through
// KaGen, lib/io/io_utils.h:72-73): n points in a disk of radius R, angle
// uniform, radius with density alpha sinh(alpha r) / (cosh(alpha R) - 1),
// alpha = (gamma - 1) / 2; u ~ w iff their hyperbolic distance is <= R.
//
// Exactness.  With a = e^r, b = e^-r, s = sinh r and p = (cos t, sin t),
//   cosh d(u, w) <= cosh R
//   <=>  |p_u - p_w|^2 * (s_u * s_w)  <=  2 cosh R - (a_u b_w + b_u a_w)
// (|p_u - p_w|^2 = 4 sin^2(dt / 2)).  Every quantity on the left and right is
// computed from per-point values with + - * / and sqrt only, each rounded
// once (the device path calls the _rn intrinsics, so no multiply-add is ever
// contracted; the host is built with -ffp-contract=off), and the per-point
// values come from exp / log / sin / cos evaluated here by fixed series with
// the same operations.  IEEE 754 rounds these operations identically on
// every host and on the GPU, so host and device take the same decision for
// every pair, and the decision is symmetric in (u, w) bit for bit: the two
// products of the cosh term and the two squares are the same numbers in
// either order, and the sums are commutative.
//
// Candidate search.  The generators only need a superset of each point's
// neighbours: points are bucketed into radial bands [k, k+1) and, per band,
// into angular cells; a point visits, in each band, the cells within the
// largest connecting angle to the band's inner edge (the connecting angle
// decreases with the other point's radius), widened by a relative 1e-5 and an
// absolute 1e-8 rad so that rounding can never hide a neighbour, and only the
// exact test above decides.  The bound itself may use the platform's asin.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define RHG_HD __host__ __device__ __forceinline__
#else
#define RHG_HD inline
#endif

#include <math.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/cc_gpu.h"

namespace rhg {

constexpr int kMaxBands = 96;

// ---- correctly rounded basic operations -------------------------------------
RHG_HD double add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
RHG_HD double sub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
RHG_HD double mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
RHG_HD double div(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
RHG_HD double sqrt_rn(double a) {
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(a);
#else
  return __builtin_sqrt(a);
#endif
}
RHG_HD uint64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
RHG_HD double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
// integer (|k| < 2^53) to double, exact
RHG_HD double i2d(int64_t k) { return (double)k; }
// 2^k for -1022 <= k <= 1023, exact
RHG_HD double pow2(int k) { return from_bits((uint64_t)(k + 1023) << 52); }

// ---- hash -------------------------------------------------------------------
RHG_HD uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
RHG_HD uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
  return mix64(mix64(mix64(seed) ^ a) ^ (b * 0xd6e8feb86659fd93ull));
}
// uniform in [0, 1): the top 53 bits, exact
RHG_HD double unit(uint64_t h) { return mul(i2d((int64_t)(h >> 11)), pow2(-53)); }

// ---- elementary functions by fixed series -----------------------------------
// Written from the Taylor series with range reduction (no libm and no CUDA
// math routine): deterministic first, accurate to a few ulp.
constexpr double kLn2 = 0.693147180559945309417232121458;
constexpr double kPi = 3.14159265358979323846264338328;

// e^x for |x| <= 700: x = k ln2 + r, |r| <= ln2 / 2, e^r by 22 Taylor terms
// (Horner), times 2^k.
RHG_HD double exp_det(double x) {
  const double kf = floor(add(div(x, kLn2), 0.5));
  const int k = (int)kf;
  const double r = sub(x, mul(kf, kLn2));
  double p = 1.0;
  for (int i = 22; i >= 1; --i) p = add(1.0, mul(div(r, i2d(i)), p));
  if (k > 1000) return mul(mul(p, pow2(1000)), pow2(k - 1000));
  if (k < -1000) return mul(mul(p, pow2(-1000)), pow2(k + 1000));
  return mul(p, pow2(k));
}

// log x for normal x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh(t), t = (m - 1) / (m + 1), |t| < 0.172, 20 odd terms.
RHG_HD double log_det(double x) {
  uint64_t u = bits_of(x);
  int e = (int)((u >> 52) & 0x7ff) - 1023;
  double m = from_bits((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);  // [1, 2)
  if (m > 1.4142135623730951) {
    m = mul(m, 0.5);
    e += 1;
  }
  const double t = div(sub(m, 1.0), add(m, 1.0));
  const double t2 = mul(t, t);
  double s = 0.0;
  for (int i = 39; i >= 3; i -= 2) s = mul(t2, add(div(1.0, i2d(i)), s));
  const double lm = mul(2.0, add(t, mul(t, s)));
  return add(mul(i2d(e), kLn2), lm);
}

// sin and cos of an angle in [0, pi/4] given as f * 2^-53 * pi/4, 0 <= f <= 2^53
RHG_HD void sincos_octant(int64_t f, double *s, double *c) {
  const double t = mul(mul(i2d(f), pow2(-53)), 0.25 * kPi);
  const double t2 = mul(t, t);
  double ps = 1.0, pc = 1.0;
  for (int i = 26; i >= 2; i -= 2) {
    ps = sub(1.0, mul(div(t2, i2d(i * (i + 1))), ps));
    pc = sub(1.0, mul(div(t2, i2d(i * (i - 1))), pc));
  }
  *s = mul(t, ps);
  *c = pc;
}

// (cos, sin) of the angle 2 pi phi / 2^64 (the top 53 bits of phi are used)
RHG_HD void cossin_phase(uint64_t phi, double *x, double *y) {
  const int oct = (int)(phi >> 61);
  const int64_t f = (int64_t)((phi << 3) >> 11);  // position in the octant, 53 bits
  double sb, cb;                                   // sin, cos of the angle within the quadrant
  if (oct & 1) {
    double s, c;
    sincos_octant(((int64_t)1 << 53) - f, &s, &c);  // pi/2 - angle
    sb = c;
    cb = s;
  } else {
    sincos_octant(f, &sb, &cb);
  }
  switch (oct >> 1) {
    case 0: *x = cb; *y = sb; break;
    case 1: *x = -sb; *y = cb; break;
    case 2: *x = -cb; *y = -sb; break;
    default: *x = sb; *y = -cb; break;
  }
}

// ---- the model --------------------------------------------------------------
// Per-graph constants, computed once on the host and passed to both paths.
struct Params {
  uint64_t n, seed;
  int idbits;        // bits of a vertex index: keys are (angle bits << idbits) | index
  int nb;            // radial bands [k, k + 1), k = 0 .. nb - 1
  double alpha, R;
  double two_cosh_R;      // 2 cosh R
  double cosh_aR_m1;      // cosh(alpha R) - 1
  double band_a[kMaxBands], band_b[kMaxBands], band_s[kMaxBands];  // e^k, e^-k, sinh k
  double band_inv4s[kMaxBands];  // 1 / (4 sinh k) (0 for k = 0), for the window bound only
};

struct Point {
  double a, b, s, x, y;  // e^r, e^-r, sinh r, cos t, sin t
  uint64_t phi;          // angle as a fraction of the full turn, 2^64 = 2 pi
  int band;
};

// The sort key of vertex index i: points are numbered in increasing angle
// (ties, impossible in practice, by index).
RHG_HD uint64_t angle_key(const Params &P, uint64_t i) {
  return ((hash3(P.seed, i, 21) >> P.idbits) << P.idbits) | i;
}

// The point with sort key `key` (angle key of its original index).
RHG_HD Point point(const Params &P, uint64_t key) {
  Point p;
  const uint64_t mask = (P.idbits >= 64) ? ~0ull : ((1ull << P.idbits) - 1);
  const uint64_t src = key & mask;
  p.phi = key & ~mask;
  cossin_phase(p.phi, &p.x, &p.y);
  // radius by the inverse CDF: cosh(alpha r) = 1 + u (cosh(alpha R) - 1)
  const double u = unit(hash3(P.seed, src, 22));
  const double z = add(1.0, mul(u, P.cosh_aR_m1));
  const double w = add(z, sqrt_rn(sub(mul(z, z), 1.0)));  // e^(alpha r)
  double r = div(log_det(w), P.alpha);
  if (r < 0.0) r = 0.0;
  p.a = exp_det(r);
  p.b = div(1.0, p.a);
  p.s = mul(sub(p.a, p.b), 0.5);
  int band = (int)floor(r);
  p.band = band < 0 ? 0 : (band >= P.nb ? P.nb - 1 : band);
  return p;
}

// u ~ w (the exact decision; symmetric bit for bit)
RHG_HD bool adjacent(const Params &P, const Point &u, const Point &w) {
  const double dx = sub(u.x, w.x), dy = sub(u.y, w.y);
  const double d2 = add(mul(dx, dx), mul(dy, dy));
  const double lhs = mul(d2, mul(u.s, w.s));
  const double rhs = sub(P.two_cosh_R, add(mul(u.a, w.b), mul(u.b, w.a)));
  return lhs <= rhs;
}

// Half-width, in phase units, of the angular window of band `band` around u
// that holds every neighbour of u in that band; returns false when the whole
// band must be scanned.
RHG_HD bool window(const Params &P, const Point &u, int band, double inv_su, uint64_t *half) {
  const double se = P.band_s[band];
  if (se <= 0.0 || u.s <= 0.0) return false;
  // q = sin^2(theta_max / 2) at the band's inner radius.  Only a bound: the
  // numerator has no cancellation for bands above the first (|r - k| <= R - 1),
  // so q is good to a few 1e-16; the angle is then taken in single precision
  // (relative error below 1e-6, well inside the widening).
  const double q = (P.two_cosh_R - (u.a * P.band_b[band] + u.b * P.band_a[band])) * inv_su *
                   P.band_inv4s[band];
  if (q >= 0.49) return false;  // theta_max >= ~88 degrees: scan the band
  const float qf = (float)(q > 0.0 ? q : 0.0) * 1.000001f;
#ifdef __CUDA_ARCH__
  const float th = 2.0f * asinf(sqrtf(qf));
#else
  const float th = 2.0f * __builtin_asinf(__builtin_sqrtf(qf));
#endif
  const double wide = (double)th * (1.0 + 1e-5) + 1e-8;  // radians
  *half = (uint64_t)(wide * (18446744073709551616.0 / (2.0 * kPi)));
  return true;
}

// Cells of a band: 2^L cells over the full turn, L = floor(log2(points / 2)).
RHG_HD int cell_bits(uint64_t band_points) {
  int L = 0;
  while (L < 40 && (2ull << (L + 1)) <= band_points) ++L;
  return L;
}
RHG_HD uint64_t cell_of(uint64_t phi, int L) { return L == 0 ? 0 : phi >> (64 - L); }

}  // namespace rhg

// ---- per-graph constants (host functions) --------------------------------------
namespace rhg {

// Expected average degree for radius R: (n - 1) * E[theta_max / pi], the
// expectation over two independent radii, with sin^2(theta_max / 2) =
// (cosh R - cosh(r1 - r2)) / (2 sinh r1 sinh r2).  Midpoint rule on a uniform
// grid in r with density weights: the few vertices near the centre have
// degrees close to n, so the grid must resolve small radii too (a grid in CDF
// space does not, and underestimates the degree).
inline double avg_degree(uint64_t n, double alpha, double R) {
  const int N = 1200;
  std::vector<double> r(N), w(N), sh(N), W(N + 1, 0.0);
  double wsum = 0.0;
  for (int i = 0; i < N; ++i) {
    r[i] = (i + 0.5) * R / N;
    w[i] = std::sinh(alpha * r[i]);
    wsum += w[i];
    W[i + 1] = W[i] + w[i];
    sh[i] = std::sinh(r[i]);
  }
  const double coshR = std::cosh(R);
  // theta is symmetric: the pairs j > i counted twice, the diagonal once; the
  // pairs with r_i + r_j <= R (a prefix of j, r ascending) all have theta = pi
  double acc = 0.0;
  for (int i = 0; i < N; ++i) {
    int jfull = (int)std::floor((R - r[i]) * N / R - 0.5);  // last j with r_j <= R - r_i
    while (jfull + 1 < N && r[i] + r[jfull + 1] <= R) ++jfull;
    while (jfull >= 0 && r[i] + r[jfull] > R) --jfull;
    double row = 0.0;
    const int j0 = i + 1;
    if (jfull >= j0) row += kPi * (W[jfull + 1] - W[j0]);
    for (int j = std::max(j0, jfull + 1); j < N; ++j) {
      const double q = (coshR - std::cosh(r[i] - r[j])) / (2.0 * sh[i] * sh[j]);
      const double th = q >= 1.0 ? kPi : (q <= 0.0 ? 0.0 : 2.0 * std::asin(std::sqrt(q)));
      row += w[j] * th;
    }
    double diag;
    if (2.0 * r[i] <= R) {
      diag = kPi;
    } else {
      const double q = (coshR - 1.0) / (2.0 * sh[i] * sh[i]);
      diag = q >= 1.0 ? kPi : (q <= 0.0 ? 0.0 : 2.0 * std::asin(std::sqrt(q)));
    }
    acc += w[i] * (2.0 * row + w[i] * diag);
  }
  return (double)(n - 1) * acc / (wsum * wsum * kPi);
}

// The radius for the target degree: a bracketed root of log avg_degree(R) -
// log deg (decreasing in R) by the Illinois variant of regula falsi, a few
// evaluations instead of forty bisection steps, then rounded to a multiple of
// 2^-32 so that the last bits of the platform's sinh / asin cannot move it.
inline double target_radius(uint64_t n, double alpha, double deg) {
  // in log space the degree falls about linearly in R (as e^(-R/2)), which
  // regula falsi solves in a few steps
  auto f = [&](double R) { return std::log(avg_degree(n, alpha, R)) - std::log(deg); };
  double lo = 1e-3, hi = 2.0 * std::log((double)n) + 40.0;
  double flo = f(lo), fhi = f(hi);
  if (!(flo > 0.0) || !(fhi < 0.0)) return std::ldexp(std::nearbyint(std::ldexp(0.5 * (lo + hi), 32)), -32);
  int side = 0;
  for (int it = 0; it < 200 && hi - lo > 1e-12 * hi; ++it) {
    double mid = (lo * fhi - hi * flo) / (fhi - flo);
    if (!(mid > lo && mid < hi)) mid = 0.5 * (lo + hi);
    const double fm = f(mid);
    if (fm == 0.0) {
      lo = hi = mid;
      break;
    }
    if (fm > 0.0) {
      lo = mid;
      flo = fm;
      if (side == 1) fhi *= 0.5;
      side = 1;
    } else {
      hi = mid;
      fhi = fm;
      if (side == -1) flo *= 0.5;
      side = -1;
    }
  }
  return std::ldexp(std::nearbyint(std::ldexp(0.5 * (lo + hi), 32)), -32);
}

inline int make_params(uint64_t n, double avg_deg, double gamma, uint64_t seed, Params *P) {
  if (n < 2 || n >= (1ull << 32) || !(gamma > 2.0) || !(avg_deg > 0.0)) return CC_ERR_INVALID;
  std::memset(P, 0, sizeof(*P));
  P->n = n;
  P->seed = seed;
  P->idbits = 1;
  while (P->idbits < 64 && (1ull << P->idbits) < n) ++P->idbits;
  P->alpha = (gamma - 1.0) / 2.0;
  P->R = target_radius(n, P->alpha, avg_deg);
  P->two_cosh_R = add(exp_det(P->R), exp_det(-P->R));
  const double aR = mul(P->alpha, P->R);
  P->cosh_aR_m1 = sub(mul(add(exp_det(aR), exp_det(-aR)), 0.5), 1.0);
  P->nb = (int)std::floor(P->R) + 1;
  if (P->nb > kMaxBands) return CC_ERR_UNSUPPORTED;
  for (int k = 0; k < P->nb; ++k) {
    P->band_a[k] = exp_det((double)k);
    P->band_b[k] = div(1.0, P->band_a[k]);
    P->band_s[k] = mul(sub(P->band_a[k], P->band_b[k]), 0.5);
    P->band_inv4s[k] = P->band_s[k] > 0.0 ? 1.0 / (4.0 * P->band_s[k]) : 0.0;
  }
  return CC_OK;
}

}  // namespace rhg

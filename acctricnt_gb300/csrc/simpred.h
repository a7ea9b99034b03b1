// Exact-integer form of the reference's SCAN similarity predicate.
//
// The reference decides entry (u,v) similar when
//     (double)((long double)cnn / sqrt((long double)du * dv)) >= eps
// (scan-query-cuda/scan_xp_common.cu:247-250, scan-query/scan_xp.cpp:119-121),
// with cnn = |N(u) ∩ N(v)| + 2 and du, dv = degree + 1.  Rounding the exact value
// x = cnn / sqrt(du*dv) to a double gives a result >= eps exactly when x lies
// above the midpoint M between eps and its predecessor double (or on M, when eps
// has an even significand: ties round to even).  M = P * 2^s with P odd, so the
// test is  cnn^2 * 2^(-2s)  >  P^2 * du * dv  (or >= on a tie-to-eps), an integer
// comparison of at most 236 bits.  A double-precision estimate decides all but a
// thin band around M; only that band takes the multi-word path.
//
// The long double intermediates of the reference (64-bit significand on x86,
// 113-bit on aarch64) can only differ from this when x lies within ~2^-62
// relative of M; for integer cnn < 2^32 and du*dv < 2^64 the tests compare the two
// on exhaustive small grids and on every entry of every test graph.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define ACCX_PHD __host__ __device__ __forceinline__
#else
#define ACCX_PHD inline
#endif

// Per-query constants, computed once on the host from eps.
struct accx_simq {
  int mode;        // 0: compare, 1: always similar, 2: never similar
  int tie_true;    // x == M counts as similar
  int shift;       // -2s, in [0, 236]
  uint64_t P;      // odd, < 2^55
  double m2_lo;    // M^2 * (1 - 2^-40): x^2 below this is certainly not similar
  double m2_hi;    // M^2 * (1 + 2^-40): x^2 above this is certainly similar
};

static inline accx_simq accx_simq_make(double eps) {
  accx_simq q;
  memset(&q, 0, sizeof(q));
  if (eps != eps) { q.mode = 2; return q; }          // NaN: every comparison false
  if (eps <= 0.0) { q.mode = 1; return q; }          // x > 0 always
  if (eps > 4294967296.0) { q.mode = 2; return q; }  // x <= cnn < 2^32
  uint64_t bits;
  memcpy(&bits, &eps, 8);
  int bexp = (int)((bits >> 52) & 0x7ff);
  uint64_t frac = bits & ((1ull << 52) - 1);
  uint64_t E;
  int k;
  if (bexp == 0) { E = frac; k = -1074; } else { E = frac | (1ull << 52); k = bexp - 1075; }
  // Midpoint between pred(eps) and eps.
  uint64_t P;
  int s;
  if (E == (1ull << 52) && bexp > 1) {  // eps a power of two above the subnormal range
    P = (1ull << 54) - 1;
    s = k - 2;
  } else {
    P = 2 * E - 1;
    s = k - 1;
  }
  q.tie_true = (E % 2 == 0);
  // x >= 2/2^32 for any valid entry (cnn >= 2, du*dv < 2^64): M below that is always met.
  double M = ldexp((double)P, s);  // rounding only matters for the fast band, not the decision
  if (M < ldexp(1.0, -33)) { q.mode = 1; return q; }
  q.mode = 0;
  q.P = P;
  q.shift = -2 * s;  // s <= -1 here because M < 2^32 needs s < 32 - 54
  double m2 = M * M;
  q.m2_lo = m2 * (1.0 - ldexp(1.0, -40));
  q.m2_hi = m2 * (1.0 + ldexp(1.0, -40));
  return q;
}

ACCX_PHD uint64_t accx_umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Exact: sign of cnn^2 * 2^shift - P^2 * D  (-1, 0, +1), 4-limb little endian.
ACCX_PHD int accx_cmp_exact(uint64_t cnn, uint64_t D, uint64_t P, int shift) {
  uint64_t c2 = cnn * cnn;  // cnn < 2^32
  uint64_t L[4] = {0, 0, 0, 0};
  int li = shift >> 6, lb = shift & 63;
  if (li < 4) L[li] = c2 << lb;
  if (lb && li + 1 < 4) L[li + 1] = c2 >> (64 - lb);
  // R = (P*P) * D, P*P < 2^110.
  uint64_t p0 = P * P, p1 = accx_umulhi(P, P);
  uint64_t r0 = p0 * D;
  uint64_t t0 = accx_umulhi(p0, D);
  uint64_t m1 = p1 * D;
  uint64_t r1 = m1 + t0;
  uint64_t carry = (r1 < m1) ? 1u : 0u;
  uint64_t r2 = accx_umulhi(p1, D) + carry;
  uint64_t R[4] = {r0, r1, r2, 0};
  for (int i = 3; i >= 0; i--) {
    if (L[i] != R[i]) return L[i] > R[i] ? 1 : -1;
  }
  return 0;
}

// cnn = count + 2, du/dv = degree + 1 (the reference's inclusive degrees).
ACCX_PHD bool accx_similar(const accx_simq &q, uint32_t cnn, uint32_t du, uint32_t dv) {
  if (q.mode != 0) return q.mode == 1;
  uint64_t D = (uint64_t)du * (uint64_t)dv;
  double c = (double)cnn;
  double x2 = (c * c) / (double)D;
  if (x2 > q.m2_hi) return true;
  if (x2 < q.m2_lo) return false;
  int s = accx_cmp_exact(cnn, D, q.P, q.shift);
  return s > 0 || (s == 0 && q.tie_true);
}

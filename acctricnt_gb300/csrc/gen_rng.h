// Counter-based random streams for the synthetic graph generators.  Every draw
// is a pure function of (seed, draw index), computed with integer operations
// only, so the host generator and the device generator emit identical edge
// streams and any thread count or launch shape gives the same graph.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ACCX_HD __host__ __device__ __forceinline__
#else
#define ACCX_HD inline
#endif

// SplitMix64 finaliser (Steele, Lea, Flood: "Fast splittable pseudorandom
// number generators", OOPSLA 2014).
ACCX_HD uint64_t accx_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

ACCX_HD uint64_t accx_draw(uint64_t seed_mix, uint64_t counter) { return accx_mix64(seed_mix + counter * 0xD1B54A32D192ED03ull); }

// floor(x * bound / 2^64) without a 128-bit type on the device.
ACCX_HD uint64_t accx_mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// R-MAT quadrant thresholds as 53-bit integers: a draw r = x >> 11 picks
// (0,0) if r < ta, (0,1) if r < tab, (1,0) if r < tabc, else (1,1).
struct accx_rmat_thresholds {
  uint64_t ta, tab, tabc;
};

// One R-MAT edge: `scale` independent quadrant choices, most significant bit first.
ACCX_HD void accx_rmat_edge(uint64_t seed_mix, uint64_t k, int scale, accx_rmat_thresholds t, uint32_t *u,
                            uint32_t *v) {
  uint32_t uu = 0, vv = 0;
  for (int j = 0; j < scale; j++) {
    uint64_t r = accx_draw(seed_mix, k * 64u + (uint64_t)j) >> 11;
    uint32_t ub = r >= t.tab ? 1u : 0u;
    uint32_t vb = ((r >= t.ta) & (r < t.tab)) | (r >= t.tabc) ? 1u : 0u;
    uu = (uu << 1) | ub;
    vv = (vv << 1) | vb;
  }
  *u = uu;
  *v = vv;
}

ACCX_HD void accx_er_edge(uint64_t seed_mix, uint64_t k, uint64_t n, uint32_t *u, uint32_t *v) {
  *u = (uint32_t)accx_mulhi64(accx_draw(seed_mix, 2 * k), n);
  *v = (uint32_t)accx_mulhi64(accx_draw(seed_mix, 2 * k + 1), n);
}

// Chung-Lu endpoint: r in [0, 2^62) mapped through the cumulative weight table
// cdf[0..n] (cdf[0] = 0, cdf[n] = 2^62): the largest i with cdf[i] <= r.
ACCX_HD uint32_t accx_cdf_pick(const uint64_t *cdf, uint64_t n, uint64_t r) {
  uint64_t lo = 0, hi = n;  // invariant: cdf[lo] <= r < cdf[hi]
  while (hi - lo > 1) {
    uint64_t mid = (lo + hi) >> 1;
    if (cdf[mid] <= r) lo = mid; else hi = mid;
  }
  return (uint32_t)lo;
}

ACCX_HD void accx_cl_edge(uint64_t seed_mix, uint64_t k, const uint64_t *cdf, uint64_t n, uint32_t *u,
                          uint32_t *v) {
  *u = accx_cdf_pick(cdf, n, accx_draw(seed_mix, 2 * k) >> 2);
  *v = accx_cdf_pick(cdf, n, accx_draw(seed_mix, 2 * k + 1) >> 2);
}

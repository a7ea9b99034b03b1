// Device helpers shared by the libaccx kernels.
#pragma once
#include <stdint.h>

#define ACCX_FULL_MASK 0xffffffffu

// Largest r in [lo, hi) with off[r] <= e.  For a CSR this is the row that holds
// entry e (rows with zero degree are skipped because off[r+1] == off[r]).
__device__ __forceinline__ uint32_t accx_row_of(const uint32_t *__restrict__ off, uint32_t lo, uint32_t hi,
                                                uint32_t e) {
  while (hi - lo > 1) {
    uint32_t mid = lo + ((hi - lo) >> 1);
    if (__ldg(off + mid) <= e) lo = mid; else hi = mid;
  }
  return lo;
}

// First index i in [b, e) with a[i] >= val (e when none).
__device__ __forceinline__ uint32_t accx_lower_bound(const int32_t *__restrict__ a, uint32_t b, uint32_t e,
                                                     int32_t val) {
  while (b < e) {
    uint32_t mid = b + ((e - b) >> 1);
    if (__ldg(a + mid) < val) b = mid + 1; else e = mid;
  }
  return b;
}

// Entry tiles: a CTA of TILE threads maps entries [base, base+TILE) to rows.
// With `tilerow` (row of every tile's first entry, built once per CSR by
// accx_tilerow_build) the CTA reads its row range; without it two threads
// search the whole offset array.  Each thread then searches only the rows the
// tile spans.  Launch one CTA per tile (blockIdx.x = tile).
template <int TILE>
struct accx_tile_rows {
  uint32_t r_lo, r_hi;
};

// The same for tile `tile` (base = tile * TILE), for CTAs that loop over tiles;
// such a loop must put a __syncthreads between two calls (sh is rewritten).
template <int TILE>
__device__ __forceinline__ uint32_t accx_tile_row_at(const uint32_t *__restrict__ off,
                                                     const uint32_t *__restrict__ tilerow, uint32_t n, uint32_t m,
                                                     uint32_t tile, uint32_t base, uint32_t e,
                                                     accx_tile_rows<TILE> *sh) {
  if (tilerow) {
    if (threadIdx.x == 0) {
      sh->r_lo = __ldg(tilerow + tile);
      sh->r_hi = __ldg(tilerow + tile + 1);
    }
  } else {
    if (threadIdx.x == 0) sh->r_lo = accx_row_of(off, 0, n, base);
    if (threadIdx.x == 1 || blockDim.x == 1) {
      uint32_t last = base + TILE - 1;
      if (last >= m) last = m - 1;
      sh->r_hi = accx_row_of(off, 0, n, last);
    }
  }
  __syncthreads();
  uint32_t r = 0;
  if (e < m) r = accx_row_of(off, sh->r_lo, sh->r_hi + 1, e);
  return r;
}

template <int TILE>
__device__ __forceinline__ uint32_t accx_tile_row(const uint32_t *__restrict__ off,
                                                  const uint32_t *__restrict__ tilerow, uint32_t n, uint32_t m,
                                                  uint32_t base, uint32_t e, accx_tile_rows<TILE> *sh) {
  return accx_tile_row_at<TILE>(off, tilerow, n, m, blockIdx.x, base, e, sh);
}

// Degree-owner rule of the reference CPU bitmap build (scan-query/scan_xp.cpp:290-292):
// u owns edge (u,v) when d_u > d_v, or d_u == d_v and u < v.
__device__ __forceinline__ bool accx_owns(uint32_t u, uint32_t du, uint32_t v, uint32_t dv) {
  return du > dv || (du == dv && u < v);
}

__device__ __forceinline__ int accx_bucket(uint32_t d) {
  int b = 31 - __clz(d | 1u);
  return b < ACCX_NB - 1 ? b : ACCX_NB - 1;
}

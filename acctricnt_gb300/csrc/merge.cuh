// Warp merge-path intersection count, shared by the counting kernels.
#pragma once
#include <stdint.h>

#include "devutil.cuh"

#define MERGE_WIN 128  // int32 per list window (32 lanes x uint4)

// Warp merge-path intersection.
//
// Each list is consumed in windows of 128 ids loaded by the 32 lanes as 16-byte
// vectors from 16-byte aligned addresses (the first window of a list starts at
// the list's first entry and may be shorter).  A window pair is intersected by
// merge path: every lane takes an equal share of the merged order (a binary
// search on its diagonal), walks it, and counts B[j] when the A element just
// before it in merged order (ties take A first) equals it.  The window whose last
// id is smaller is then replaced (both on equality); matches cannot straddle a
// replaced window, so every common id is counted exactly once.
__device__ __forceinline__ int accx_load_window(const int32_t *__restrict__ dst, uint32_t pos, uint32_t end,
                                                int32_t *__restrict__ buf, int lane) {
  uint32_t al = pos & ~3u;
  uint32_t idx = al + 4u * (uint32_t)lane;
  if (idx < end && idx + 4u > pos) {
    int4 q = __ldg(reinterpret_cast<const int4 *>(dst + idx));
    int32_t vals[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int t = 0; t < 4; t++) {
      uint32_t ii = idx + (uint32_t)t;
      if (ii >= pos && ii < end) buf[ii - pos] = vals[t];
    }
  }
  uint32_t lim = al + MERGE_WIN;
  if (lim > end) lim = end;
  return (int)(lim - pos);
}

__device__ __forceinline__ uint32_t accx_warp_merge_count(const int32_t *__restrict__ dst, uint32_t ab, uint32_t ae,
                                                          uint32_t bb, uint32_t be, int32_t *__restrict__ A,
                                                          int32_t *__restrict__ B, int lane) {
  uint32_t c = 0;
  if (ab >= ae || bb >= be) return 0;
  int la = accx_load_window(dst, ab, ae, A, lane);
  int lb = accx_load_window(dst, bb, be, B, lane);
  __syncwarp();
  for (;;) {
    int32_t a_first = A[0], a_last = A[la - 1], b_first = B[0], b_last = B[lb - 1];
    if (a_last >= b_first && b_last >= a_first) {
      int total = la + lb;
      int chunk = (total + 31) >> 5;
      int d0 = min(lane * chunk, total), d1 = min(d0 + chunk, total);
      int lo = max(0, d0 - lb), hi = min(d0, la);
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (A[mid] <= B[d0 - mid - 1]) lo = mid + 1; else hi = mid;
      }
      int i = lo, j = d0 - lo;
      for (int d = d0; d < d1; d++) {
        if (i < la && (j >= lb || A[i] <= B[j])) {
          i++;
        } else {
          if (i > 0 && A[i - 1] == B[j]) c++;
          j++;
        }
      }
    }
    bool adv_a = a_last <= b_last, adv_b = b_last <= a_last;
    __syncwarp();
    if (adv_a) {
      ab += (uint32_t)la;
      if (ab >= ae) break;
      la = accx_load_window(dst, ab, ae, A, lane);
    }
    if (adv_b) {
      bb += (uint32_t)lb;
      if (bb >= be) break;
      lb = accx_load_window(dst, bb, be, B, lane);
    }
    __syncwarp();
  }
  return __reduce_add_sync(ACCX_FULL_MASK, c);
}


// The same walk for oriented counting: every common id is a triangle, and the
// two entries that hold it (its position in list A and in list B) each get +1
// in cnt (fire-and-forget atomics; other triangles credit the same entries).
// Returns the number of common ids (the triangle credit of the edge itself).
__device__ __forceinline__ uint32_t accx_warp_merge_credit(const int32_t *__restrict__ dst, uint32_t ab, uint32_t ae,
                                                           uint32_t bb, uint32_t be, int32_t *__restrict__ A,
                                                           int32_t *__restrict__ B, int lane,
                                                           int32_t *__restrict__ cnt) {
  uint32_t c = 0;
  if (ab >= ae || bb >= be) return 0;
  int la = accx_load_window(dst, ab, ae, A, lane);
  int lb = accx_load_window(dst, bb, be, B, lane);
  __syncwarp();
  for (;;) {
    int32_t a_first = A[0], a_last = A[la - 1], b_first = B[0], b_last = B[lb - 1];
    if (a_last >= b_first && b_last >= a_first) {
      int total = la + lb;
      int chunk = (total + 31) >> 5;
      int d0 = min(lane * chunk, total), d1 = min(d0 + chunk, total);
      int lo = max(0, d0 - lb), hi = min(d0, la);
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (A[mid] <= B[d0 - mid - 1]) lo = mid + 1; else hi = mid;
      }
      int i = lo, j = d0 - lo;
      for (int d = d0; d < d1; d++) {
        if (i < la && (j >= lb || A[i] <= B[j])) {
          i++;
        } else {
          if (i > 0 && A[i - 1] == B[j]) {
            c++;
            atomicAdd(cnt + ab + (uint32_t)(i - 1), 1);
            atomicAdd(cnt + bb + (uint32_t)j, 1);
          }
          j++;
        }
      }
    }
    bool adv_a = a_last <= b_last, adv_b = b_last <= a_last;
    __syncwarp();
    if (adv_a) {
      ab += (uint32_t)la;
      if (ab >= ae) break;
      la = accx_load_window(dst, ab, ae, A, lane);
    }
    if (adv_b) {
      bb += (uint32_t)lb;
      if (bb >= be) break;
      lb = accx_load_window(dst, bb, be, B, lane);
    }
    __syncwarp();
  }
  return __reduce_add_sync(ACCX_FULL_MASK, c);
}

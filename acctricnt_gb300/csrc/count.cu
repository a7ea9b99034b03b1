// All-edge common-neighbour counting on sm_103a.
//
// What it computes is the reference's CheckCore output (common_node_num[e] =
// 2 + |N(u) ∩ N(v)| for every CSR entry; scan-query-cuda/scan_xp_common.cu:24-39,
// :220-237 and the kernels in scan_xp_multi_gpu_multi_pass_common.cu:32-495).
// How it computes it:
//   * every undirected edge is counted once, by its owner -- the endpoint with
//     the larger degree (ties: smaller id), the rule of the reference CPU bitmap
//     build (scan-query/scan_xp.cpp:290-292) -- so the probed list is always the
//     shorter one; the reference GPU kernels use u < v instead;
//   * a classify pass sorts owned edges into three kernels by a per-degree-bucket
//     policy (the reference's fixed ratio-50 rule, a table, or the trained cost
//     model): warp merge-path, galloping binary search, or a per-owner
//     shared-memory bitmap;
//   * a mirror pass writes the count of the reverse entry (u found in N(v) by
//     binary search), which replaces the reference's CPU reverse-offset
//     co-routine and PostComputeCoreChecking copy
//     (experimental_scan_xp_multigpu_multipass.cu:6-23, scan_xp_common.cu:223-233).
// No launch needs a host round trip: list lengths live in device counters and
// the counting kernels are persistent grid-stride loops, so a whole count is a
// fixed sequence of launches on one stream (capturable in a CUDA graph).
#include <string.h>

#include "accx_internal.h"
#include "devutil.cuh"

// counters layout
#define C_MERGE 0
#define C_GALLOP 1
#define C_ITEMS 2
#define C_EDGES 3  // + kind
#define C_WORK 6   // + kind
#define C_OWNER 9  // + kind: owner-side elements
#define C_NUM 16

#define MERGE_WIN 128        // int32 per list window (32 lanes x uint4)
#define MERGE_WARPS 8        // warps per merge/gallop CTA
#define ITEM_TARGET_DEFAULT (1u << 17)  // probe elements per bitmap work item

// Kind of an owned edge; du = owner degree >= dv.
__device__ __forceinline__ int accx_edge_kind(int policy, const uint8_t *table, uint32_t du, uint32_t dv) {
  switch (policy) {
    case ACCX_POLICY_HEURISTIC:
      // reference GPU rule: skew_ratio * d_small < d_large -> galloping, ratio 50
      // (scan_xp_multi_gpu_multi_pass_common.cu:57-59, :105-107)
      return (50ull * dv < (unsigned long long)du) ? ACCX_KIND_GALLOP : ACCX_KIND_MERGE;
    case ACCX_POLICY_MERGE: return ACCX_KIND_MERGE;
    case ACCX_POLICY_GALLOP: return ACCX_KIND_GALLOP;
    case ACCX_POLICY_BITMAP: return ACCX_KIND_BITMAP;
    default: return table[accx_bucket(du) * ACCX_NB + accx_bucket(dv)];
  }
}

// ---------------------------------------------------------------------------
// classify: one thread per CSR entry.
template <int TILE>
__global__ void __launch_bounds__(TILE) k_classify(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                                   uint32_t n, uint32_t m, int policy,
                                                   const uint8_t *__restrict__ table, uint2 *__restrict__ list,
                                                   uint32_t list_cap, unsigned long long *__restrict__ work_u,
                                                   unsigned long long *__restrict__ ctr) {
  __shared__ accx_tile_rows<TILE> sh;
  __shared__ uint8_t s_table[ACCX_NB * ACCX_NB];
  if (policy == ACCX_POLICY_TABLE || policy == ACCX_POLICY_MODEL)
    for (int i = threadIdx.x; i < ACCX_NB * ACCX_NB; i += TILE) s_table[i] = table[i];
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, n, m, base, e, &sh);  // contains __syncthreads
  int kind = -1;
  uint32_t v = 0, du = 0, dv = 0;
  if (e < m) {
    v = (uint32_t)dst[e];
    du = off[u + 1] - off[u];
    dv = off[v + 1] - off[v];
    if (accx_owns(u, du, v, dv)) kind = accx_edge_kind(policy, s_table, du, dv);
  }
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < ACCX_NUM_KINDS; k++) {
    unsigned mask = __ballot_sync(ACCX_FULL_MASK, kind == k);
    if (!mask) continue;
    unsigned long long w = (kind == k) ? dv : 0;
    w = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)w);
    unsigned long long wo = (kind == k && k != ACCX_KIND_BITMAP) ? du : 0;
    wo = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)wo);
    int leader = __ffs(mask) - 1;
    unsigned long long basepos = 0;
    if (lane == leader) {
      atomicAdd(&ctr[C_EDGES + k], (unsigned long long)__popc(mask));
      atomicAdd(&ctr[C_WORK + k], w);
      if (wo) atomicAdd(&ctr[C_OWNER + k], wo);
      if (k == ACCX_KIND_MERGE) basepos = atomicAdd(&ctr[C_MERGE], (unsigned long long)__popc(mask));
      if (k == ACCX_KIND_GALLOP) basepos = atomicAdd(&ctr[C_GALLOP], (unsigned long long)__popc(mask));
    }
    basepos = __shfl_sync(ACCX_FULL_MASK, basepos, leader);
    if (kind == k) {
      uint32_t rank = __popc(mask & lt);
      // owned edges number exactly m/2 on a symmetric graph; the guards only
      // keep unvalidated asymmetric input inside the list
      unsigned long long idx = basepos + rank;
      if (idx < list_cap) {
        if (k == ACCX_KIND_MERGE) list[idx] = make_uint2(u, e);
        else if (k == ACCX_KIND_GALLOP) list[list_cap - 1 - idx] = make_uint2(u, e);
      }
    }
    if (k == ACCX_KIND_BITMAP && kind == k) {
      // aggregate the owner's probe work per row before the atomic
      unsigned peers = __match_any_sync(mask, u);
      unsigned sw = __reduce_add_sync(peers, dv);
      if (lane == __ffs(peers) - 1) atomicAdd(&work_u[u], (unsigned long long)sw + 1ull);
    }
  }
}

// Bitmap work items: split each bitmap owner's entry range into chunks of about
// ITEM_TARGET probe elements (at least 64 entries per chunk).
__global__ void k_make_items(const uint32_t *__restrict__ off, uint32_t n, unsigned long long *__restrict__ work_u,
                             accx_bitmap_item *__restrict__ items, unsigned long long item_cap, uint32_t target,
                             unsigned long long *__restrict__ ctr) {
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    unsigned long long w = work_u[u];
    if (!w) continue;
    work_u[u] = 0;
    uint32_t b = off[u], e = off[u + 1], d = e - b;
    unsigned long long k = (w + d + target - 1) / target;
    unsigned long long kmax = (d + 63) / 64;
    if (k > kmax) k = kmax;
    if (k < 1) k = 1;
    unsigned long long p = atomicAdd(&ctr[C_ITEMS], k);
    atomicAdd(&ctr[C_OWNER + ACCX_KIND_BITMAP], (unsigned long long)d * k);
    for (unsigned long long c = 0; c < k && p + c < item_cap; c++) {
      accx_bitmap_item it;
      it.u = u;
      it.e0 = b + (uint32_t)((unsigned long long)d * c / k);
      it.e1 = b + (uint32_t)((unsigned long long)d * (c + 1) / k);
      it.pad = 0;
      items[p + c] = it;
    }
  }
}

// ---------------------------------------------------------------------------
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

__global__ void __launch_bounds__(MERGE_WARPS * 32) k_merge(const uint32_t *__restrict__ off,
                                                             const int32_t *__restrict__ dst,
                                                             const uint2 *__restrict__ list, uint32_t list_cap,
                                                             const unsigned long long *__restrict__ ctr,
                                                             int32_t *__restrict__ cnt) {
  __shared__ __align__(16) int32_t buf[MERGE_WARPS][2][MERGE_WIN];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long total = ctr[C_MERGE];
  if (total > list_cap) total = list_cap;
  const unsigned long long nw = (unsigned long long)gridDim.x * MERGE_WARPS;
  for (unsigned long long it = (unsigned long long)blockIdx.x * MERGE_WARPS + w; it < total; it += nw) {
    uint2 p = list[it];
    uint32_t u = p.x, e = p.y;
    uint32_t v = (uint32_t)dst[e];
    uint32_t c = accx_warp_merge_count(dst, off[u], off[u + 1], off[v], off[v + 1], buf[w][0], buf[w][1], lane);
    if (lane == 0) cnt[e] = (int32_t)c;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Galloping: the owner's list A is the long one; lanes take the short list's
// ids in order and binary-search each in A.  After every round the search range
// starts at the position the last lane reached (the short list is sorted).
__global__ void __launch_bounds__(MERGE_WARPS * 32) k_gallop(const uint32_t *__restrict__ off,
                                                              const int32_t *__restrict__ dst,
                                                              const uint2 *__restrict__ list, uint32_t list_cap,
                                                              const unsigned long long *__restrict__ ctr,
                                                              int32_t *__restrict__ cnt) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long total = ctr[C_GALLOP];
  if (total > list_cap) total = list_cap;
  const unsigned long long nw = (unsigned long long)gridDim.x * MERGE_WARPS;
  for (unsigned long long it = (unsigned long long)blockIdx.x * MERGE_WARPS + w; it < total; it += nw) {
    uint2 p = list[list_cap - 1 - it];
    uint32_t u = p.x, e = p.y;
    uint32_t v = (uint32_t)dst[e];
    uint32_t ab = off[u], ae = off[u + 1], bb = off[v], be = off[v + 1];
    uint32_t c = 0;
    uint32_t lo = ab;
    for (uint32_t j0 = bb; j0 < be; j0 += 32) {
      uint32_t j = j0 + (uint32_t)lane;
      uint32_t pos = ae;
      if (j < be) {
        int32_t x = __ldg(dst + j);
        pos = accx_lower_bound(dst, lo, ae, x);
        if (pos < ae && __ldg(dst + pos) == x) c++;
      }
      // the last active lane's position bounds the next round from below
      uint32_t last_lane = (be - j0 >= 32) ? 31u : (be - j0 - 1);
      lo = __shfl_sync(ACCX_FULL_MASK, pos, (int)last_lane);
      if (lo >= ae) break;
    }
    c = __reduce_add_sync(ACCX_FULL_MASK, c);
    if (lane == 0) cnt[e] = (int32_t)c;
  }
}

// ---------------------------------------------------------------------------
// Per-owner shared-memory bitmap.
//
// A CTA takes a work item (owner u, a slice [e0,e1) of its entries).  The id
// space is cut into windows of WB ids (WB = 8 x the bitmap bytes); for every
// window that holds part of N(u) the CTA sets those bits in shared memory, then
// each warp takes an owned bitmap-kind entry (u,v), finds where N(v) enters the
// window (binary search), streams N(v) 32 ids at a time, tests the bits and
// counts hits with ballot/popc, adds the window's count to cnt[e], and the CTA
// clears the bits it set.  The reference keeps one n-bit bitmap per resident
// block in global memory and claims it with a CAS spin on per-SM slots
// (scan_xp_multi_gpu_multi_pass_common.cu:308-407); here nothing is shared
// between CTAs and nothing spins.
__global__ void k_bitmap(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst, int policy,
                         const uint8_t *__restrict__ table, const accx_bitmap_item *__restrict__ items,
                         unsigned long long item_cap, const unsigned long long *__restrict__ ctr,
                         uint32_t win_words, int32_t *__restrict__ cnt) {
  extern __shared__ __align__(16) uint32_t bm[];
  __shared__ uint8_t s_table[ACCX_NB * ACCX_NB];
  __shared__ uint32_t s_wend;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const uint32_t WB = win_words * 32u;
  for (int i = tid; i < ACCX_NB * ACCX_NB; i += nt) s_table[i] = table ? table[i] : 0;
  for (uint32_t i = tid; i < win_words; i += nt) bm[i] = 0;
  __syncthreads();
  unsigned long long total = ctr[C_ITEMS];
  if (total > item_cap) total = item_cap;
  for (unsigned long long it = blockIdx.x; it < total; it += gridDim.x) {
    accx_bitmap_item item = items[it];
    const uint32_t u = item.u;
    const uint32_t ub = off[u], ue = off[u + 1], du = ue - ub;
    uint32_t pos = ub;
    while (pos < ue) {
      const uint32_t wlo = ((uint32_t)__ldg(dst + pos) / WB) * WB;
      const uint32_t whi = wlo + WB;  // may wrap only past 2^32 ids, impossible for int32 ids
      if (tid == 0) s_wend = accx_lower_bound(dst, pos, ue, (int32_t)min(whi, 0x7fffffffu));
      __syncthreads();
      const uint32_t wend = (whi > 0x7fffffffu) ? ue : s_wend;
      for (uint32_t i = pos + tid; i < wend; i += nt) {
        uint32_t x = (uint32_t)__ldg(dst + i) - wlo;
        if (x < WB) atomicOr(&bm[x >> 5], 1u << (x & 31));  // always true for sorted rows
      }
      __syncthreads();
      for (uint32_t k = item.e0 + warp; k < item.e1; k += nwarps) {
        const uint32_t v = (uint32_t)__ldg(dst + k);
        const uint32_t vb = __ldg(off + v), ve = __ldg(off + v + 1), dv = ve - vb;
        if (dv == 0 || !accx_owns(u, du, v, dv) || accx_edge_kind(policy, s_table, du, dv) != ACCX_KIND_BITMAP)
          continue;
        if (__ldg(dst + ve - 1) < (int32_t)wlo || __ldg(dst + vb) >= (int32_t)min(whi, 0x7fffffffu)) continue;
        uint32_t s = accx_lower_bound(dst, vb, ve, (int32_t)wlo);
        uint32_t c = 0;
        for (uint32_t j0 = s; j0 < ve; j0 += 32) {
          uint32_t j = j0 + (uint32_t)lane;
          uint32_t x = (j < ve) ? (uint32_t)__ldg(dst + j) : 0xffffffffu;
          bool inwin = x < whi && x >= wlo;
          bool hit = inwin && ((bm[(x - wlo) >> 5] >> ((x - wlo) & 31)) & 1u);
          c += __popc(__ballot_sync(ACCX_FULL_MASK, hit));
          if (__ballot_sync(ACCX_FULL_MASK, !inwin)) break;
        }
        if (lane == 0 && c) cnt[k] += (int32_t)c;
      }
      __syncthreads();
      if (wend - pos > win_words / 8) {
        for (uint32_t i = tid; i < win_words; i += nt) bm[i] = 0;
      } else {
        for (uint32_t i = pos + tid; i < wend; i += nt) {
          uint32_t x = (uint32_t)__ldg(dst + i) - wlo;
          if (x < WB) bm[x >> 5] = 0;
        }
      }
      __syncthreads();
      pos = wend;
    }
  }
}

// ---------------------------------------------------------------------------
// Mirror: each owned entry e=(u,v) adds the bias and copies its count to the
// reverse entry (the position of u in N(v)).
template <int TILE>
__global__ void __launch_bounds__(TILE) k_mirror(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                                 uint32_t n, uint32_t m, int32_t bias, int32_t *__restrict__ cnt) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, n, m, base, e, &sh);
  if (e >= m) return;
  uint32_t v = (uint32_t)dst[e];
  uint32_t du = off[u + 1] - off[u];
  uint32_t vb = off[v], ve = off[v + 1];
  if (!accx_owns(u, du, v, ve - vb)) return;
  uint32_t r = accx_lower_bound(dst, vb, ve, (int32_t)u);
  int32_t c = cnt[e] + bias;
  cnt[e] = c;
  if (r < ve && dst[r] == (int32_t)u) cnt[r] = c;
}

// ---------------------------------------------------------------------------
int accx_ensure_count_scratch(accx_graph *g) {
  const size_t m = g->m, n = g->n;
  if (!g->d_cnt) ACCX_CUDA_TRY(cudaMalloc(&g->d_cnt, sizeof(int32_t) * (m ? m : 1)));
  if (!g->d_edge_list) ACCX_CUDA_TRY(cudaMalloc(&g->d_edge_list, sizeof(uint2) * (m / 2 + 1)));
  if (!g->d_items) {
    g->items_cap = n + m / 64 + 1;
    ACCX_CUDA_TRY(cudaMalloc(&g->d_items, sizeof(accx_bitmap_item) * g->items_cap));
  }
  if (!g->d_counters) {
    // counters followed by the per-vertex bitmap work array
    ACCX_CUDA_TRY(cudaMalloc(&g->d_counters, sizeof(unsigned long long) * (C_NUM + n + 1)));
    ACCX_CUDA_TRY(cudaMemset(g->d_counters, 0, sizeof(unsigned long long) * (C_NUM + n + 1)));
  }
  if (!g->d_table) ACCX_CUDA_TRY(cudaMalloc(&g->d_table, ACCX_NB * ACCX_NB));
  return ACCX_OK;
}

// Tuned defaults (overridable per call).
static int g_block_warps = 32;
static int g_window_kb = 192;


static int launch_count(accx_graph *g, const accx_count_opts *o, cudaStream_t s) {
  const uint32_t n = g->n, m = (uint32_t)g->m;
  int policy = o ? o->policy : ACCX_POLICY_HEURISTIC;
  int32_t bias = o ? o->bias : 0;
  int warps = (o && o->block_warps > 0) ? o->block_warps : g_block_warps;
  int wkb = (o && o->bitmap_window_kb > 0) ? o->bitmap_window_kb : g_window_kb;
  if (policy < ACCX_POLICY_HEURISTIC || policy > ACCX_POLICY_MODEL) return ACCX_ERR_INVALID_ARG;
  if (warps < 1 || warps > 32 || wkb < 1 || wkb > 224) return ACCX_ERR_INVALID_ARG;
  int rc = accx_ensure_count_scratch(g);
  if (rc) return rc;
  if (policy == ACCX_POLICY_TABLE) {
    if (!o->table) return ACCX_ERR_INVALID_ARG;
    for (int i = 0; i < ACCX_NB * ACCX_NB; i++)
      if (o->table[i] >= ACCX_NUM_KINDS) return ACCX_ERR_INVALID_ARG;
    ACCX_CUDA_TRY(cudaMemcpyAsync(g->d_table, o->table, ACCX_NB * ACCX_NB, cudaMemcpyHostToDevice, s));
    ACCX_CUDA_TRY(cudaStreamSynchronize(s));  // o->table is pageable caller memory
  } else if (policy == ACCX_POLICY_MODEL) {
    uint8_t t[ACCX_NB * ACCX_NB];
    rc = accx_model_table(g, t);
    if (rc) return rc;
    ACCX_CUDA_TRY(cudaMemcpyAsync(g->d_table, t, ACCX_NB * ACCX_NB, cudaMemcpyHostToDevice, s));
    ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  }
  unsigned long long *ctr = g->d_counters;
  unsigned long long *work_u = g->d_counters + C_NUM;
  ACCX_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long) * C_NUM, s));
  ACCX_CUDA_TRY(cudaMemsetAsync(g->d_cnt, 0, sizeof(int32_t) * (size_t)(m ? m : 1), s));
  if (m == 0) {
    g->cnt_bias = bias;
    g->cnt_valid = true;
    return ACCX_OK;
  }
  const uint32_t list_cap = m / 2 + 1;
  const uint32_t tiles = (m + 255) / 256;
  const bool timing = o && o->timing;
  if (timing && !g->ev[0])
    for (int i = 0; i <= ACCX_NUM_PHASES; i++) ACCX_CUDA_TRY(cudaEventCreate(&g->ev[i]));
  g->timed = timing;
#define ACCX_MARK(i) \
  if (timing) ACCX_CUDA_TRY(cudaEventRecord(g->ev[i], s));
  ACCX_MARK(0);
  k_classify<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_dst, n, m, policy, g->d_table, g->d_edge_list, list_cap,
                                        work_u, ctr);
  const int sms = accx_sm_count(g->device);
  k_make_items<<<sms * 4, 256, 0, s>>>(g->d_off, n, work_u, g->d_items, g->items_cap, ITEM_TARGET_DEFAULT, ctr);
  ACCX_MARK(1);
  k_merge<<<sms * 8, MERGE_WARPS * 32, 0, s>>>(g->d_off, g->d_dst, g->d_edge_list, list_cap, ctr, g->d_cnt);
  ACCX_MARK(2);
  k_gallop<<<sms * 8, MERGE_WARPS * 32, 0, s>>>(g->d_off, g->d_dst, g->d_edge_list, list_cap, ctr, g->d_cnt);
  ACCX_MARK(3);
  const uint32_t win_words = (uint32_t)wkb * 256u;  // KiB -> 32-bit words
  const size_t smem = (size_t)win_words * 4u;
  ACCX_CUDA_TRY(cudaFuncSetAttribute(k_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  ACCX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bitmap, warps * 32, smem));
  if (per_sm < 1) return ACCX_ERR_INVALID_ARG;
  k_bitmap<<<sms * per_sm, warps * 32, smem, s>>>(g->d_off, g->d_dst, policy, g->d_table, g->d_items, g->items_cap, ctr,
                                                  win_words, g->d_cnt);
  ACCX_MARK(4);
  k_mirror<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_dst, n, m, bias, g->d_cnt);
  ACCX_MARK(5);
#undef ACCX_MARK
  ACCX_CUDA_TRY(cudaGetLastError());
  g->cnt_bias = bias;
  g->cnt_valid = true;
  g->query_valid = false;
  g->pairs_valid = false;
  return ACCX_OK;
}

extern "C" int accx_cn_count(accx_graph *g, const accx_count_opts *opts, int32_t *out, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  ACCX_CUDA_TRY(cudaSetDevice(g->device));
  int rc = launch_count(g, opts, s);
  if (rc) {
    g->cnt_valid = false;
    return rc;
  }
  if (out) {
    rc = accx_copy_out(out, g->d_cnt, sizeof(int32_t) * (size_t)g->m, s);
    if (rc) return rc;
  }
  return ACCX_OK;
}

extern "C" int accx_cn_last_stats(const accx_graph *g, uint64_t edges[ACCX_NUM_KINDS], uint64_t work[ACCX_NUM_KINDS]) {
  if (!g || !g->d_counters) return ACCX_ERR_INVALID_ARG;
  unsigned long long h[C_NUM];
  ACCX_CUDA_TRY(cudaDeviceSynchronize());
  ACCX_CUDA_TRY(cudaMemcpy(h, g->d_counters, sizeof(h), cudaMemcpyDeviceToHost));
  for (int k = 0; k < ACCX_NUM_KINDS; k++) {
    if (edges) edges[k] = h[C_EDGES + k];
    if (work) work[k] = h[C_WORK + k];
  }
  return ACCX_OK;
}

extern "C" int accx_cn_last_owner_work(const accx_graph *g, uint64_t owner_work[ACCX_NUM_KINDS]) {
  if (!g || !g->d_counters || !owner_work) return ACCX_ERR_INVALID_ARG;
  unsigned long long h[C_NUM];
  ACCX_CUDA_TRY(cudaDeviceSynchronize());
  ACCX_CUDA_TRY(cudaMemcpy(h, g->d_counters, sizeof(h), cudaMemcpyDeviceToHost));
  for (int k = 0; k < ACCX_NUM_KINDS; k++) owner_work[k] = h[C_OWNER + k];
  return ACCX_OK;
}

extern "C" int accx_cn_last_timings(const accx_graph *g, float ms[ACCX_NUM_PHASES]) {
  if (!g || !ms) return ACCX_ERR_INVALID_ARG;
  if (!g->timed || !g->ev[0]) return ACCX_ERR_NOT_READY;
  ACCX_CUDA_TRY(cudaEventSynchronize(g->ev[ACCX_NUM_PHASES]));
  for (int i = 0; i < ACCX_NUM_PHASES; i++) ACCX_CUDA_TRY(cudaEventElapsedTime(&ms[i], g->ev[i], g->ev[i + 1]));
  return ACCX_OK;
}

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

#include <cub/cub.cuh>

#include "accx_internal.h"
#include "devutil.cuh"
#include "merge.cuh"

// counters layout
#define C_MERGE 0
#define C_GALLOP 1
#define C_ITEMS 2
#define C_EDGES 3  // + kind
#define C_WORK 6   // + kind
#define C_OWNER 9  // + kind: owner-side elements
#define C_MATCH 12 // + kind: common ids found (oriented counts)
#define C_PROBED 15 // ids probed by the oriented bitmap kernel
#define C_NUM 16

#define MERGE_WARPS 8        // warps per merge/gallop CTA
#define ITEM_TARGET_DEFAULT (1u << 20)  // probe elements per bitmap work item

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
// classify: the kind of every owned entry.  ORIENT: owners, buckets and kinds use
// the prefix lengths pre[] in place of degrees; an edge whose smaller prefix is
// empty closes no triangle from here and is left out; bitmap owners need an id
// below bm_idlim (their prefix ids fit the dense window) and a prefix of at most
// bm_pcap ids (the shared counters), otherwise their edges gallop (the lanes
// binary-search the partner's short prefix in the owner's; measured faster than
// the warp merge for these low-degree owners at every degree ratio tried).
//
// CTAs loop over blocks of 256 x CL_EPT entries; a thread takes CL_EPT
// consecutive entries, so it searches one row (inside its 256-entry tile, whose
// row range tilerow[] holds: no barrier) and follows the rows from there.  Per
// kind statistics stay in the thread's registers until the end; the bitmap
// owners' probe work is summed per row run, then per warp, before the atomic on
// work_u; merge / gallop list slots are reserved with one device atomic per list
// and block (a CTA scan of the threads' counts).
#define CL_EPT 8
// partner ranges of galloping entries carry this flag in their length (the
// bitmap kernel skips them); prefix lengths stay below 2^31 on a symmetric CSR
#define OR_SL_GALLOP 0x80000000u
struct cl_stats {
  unsigned long long e[ACCX_NUM_KINDS] = {0, 0, 0}, w[ACCX_NUM_KINDS] = {0, 0, 0}, o[ACCX_NUM_KINDS] = {0, 0, 0};
  __device__ __forceinline__ void add(int kind, uint32_t dv, uint32_t du) {
#pragma unroll
    for (int k = 0; k < ACCX_NUM_KINDS; k++)
      if (kind == k) {
        e[k]++;
        w[k] += dv;
        if (k != ACCX_KIND_BITMAP) o[k] += du;
      }
  }
};

template <bool ORIENT>
__global__ void __launch_bounds__(256, 4) k_classify(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow,
                                                  const int32_t *__restrict__ dst, uint32_t n, uint32_t m, int policy,
                                                  const uint8_t *__restrict__ table, uint2 *__restrict__ list,
                                                  uint32_t list_cap, unsigned long long *__restrict__ work_u,
                                                  unsigned long long *__restrict__ ctr, const uint32_t *__restrict__ pre,
                                                  uint32_t bm_idlim, uint32_t bm_pcap, uint2 *__restrict__ or_sl,
                                                  const uint32_t *__restrict__ rev, int32_t *__restrict__ fill,
                                                  int32_t bias, const uint2 *__restrict__ vinfo) {
  static_assert(256 % CL_EPT == 0, "chunks inside tile-row tiles");
  __shared__ uint8_t s_table[ACCX_NB * ACCX_NB];
  __shared__ uint32_t s_wc[2][8];              // per-warp merge / gallop entries of the block
  __shared__ unsigned long long s_base[2];     // the block's first slot in each list
  __shared__ unsigned long long s_st[3 * ACCX_NUM_KINDS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < 3 * ACCX_NUM_KINDS) s_st[tid] = 0;
  if (policy == ACCX_POLICY_TABLE || policy == ACCX_POLICY_MODEL)
    for (int i = tid; i < ACCX_NB * ACCX_NB; i += 256) s_table[i] = table[i];
  __syncthreads();
  cl_stats st;
  const uint32_t span = 256u * CL_EPT;
  const uint32_t nblk = (uint32_t)(((unsigned long long)m + span - 1) / span);
  for (uint32_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const uint32_t e0 = blk * span + (uint32_t)tid * CL_EPT;
    uint32_t e1 = e0 + CL_EPT < m ? e0 + CL_EPT : m;
    if (e0 >= m) e1 = e0;
    uint32_t uu[CL_EPT];
    uint32_t kinds = 0;            // 4 bits per entry (0xf: none)
    uint32_t cm = 0, cg = 0;       // this thread's merge / gallop entries
    uint32_t run_u = 0xffffffffu;  // the current row's bitmap work
    unsigned long long run_w = 0;
    if (fill && e0 < e1) {  // oriented counts start every entry at the bias
      if (e1 - e0 == CL_EPT) {
        const int4 b4 = make_int4(bias, bias, bias, bias);
        reinterpret_cast<int4 *>(fill + e0)[0] = b4;  // e0 is a multiple of 8: 32-byte aligned
        reinterpret_cast<int4 *>(fill + e0)[1] = b4;
      } else {
        for (uint32_t e = e0; e < e1; e++) fill[e] = bias;
      }
    }
    if (e0 < e1) {
      // the partners and their sizes first (independent loads in flight)
      // (oriented: the partner's offset and prefix length from one 8-byte record)
      uint32_t vv[CL_EPT], dd[CL_EPT], ss[CL_EPT];
#pragma unroll
      for (int j = 0; j < CL_EPT; j++) vv[j] = e0 + j < e1 ? (uint32_t)__ldg(dst + e0 + j) : 0u;
#pragma unroll
      for (int j = 0; j < CL_EPT; j++) {
        if (ORIENT) {
          const uint2 vi = __ldg(vinfo + vv[j]);
          ss[j] = vi.x;
          dd[j] = vi.y;
        } else {
          ss[j] = 0;
          dd[j] = __ldg(off + vv[j] + 1) - __ldg(off + vv[j]);
        }
      }
      const uint32_t t = e0 / 256u;
      uint32_t u = accx_row_of(off, __ldg(tilerow + t), __ldg(tilerow + t + 1) + 1, e0);
      uint32_t rb = __ldg(off + u), re = __ldg(off + u + 1);
      uint32_t du = ORIENT ? __ldg(pre + u) : re - rb;
#pragma unroll
      for (int j = 0; j < CL_EPT; j++) {
        const uint32_t e = e0 + (uint32_t)j;
        uu[j] = u;
        if (e >= e1) {
          kinds |= 0xfu << (4 * j);
          continue;
        }
        while (re <= e) {  // the next non-empty row
          u++;
          rb = re;
          re = __ldg(off + u + 1);
          du = ORIENT ? __ldg(pre + u) : re - rb;
        }
        uu[j] = u;
        const uint32_t v = vv[j];
        int kind = -1;
        const uint32_t dv = dd[j];
        if (ORIENT) {
          if (dv > 0 && accx_owns(u, du, v, dv)) {
            kind = accx_edge_kind(policy, s_table, du, dv);
            // outside the window or the owner counters: galloping
            if (kind == ACCX_KIND_BITMAP && (u >= bm_idlim || du > bm_pcap)) kind = ACCX_KIND_GALLOP;
          }
        } else {
          if (accx_owns(u, du, v, dv)) kind = accx_edge_kind(policy, s_table, du, dv);
        }
        uint32_t bwork = dv;
        if (ORIENT) {
          // oriented bitmap and galloping entries: the partner's prefix start and
          // its length cut at min(u, v) (galloping ones flagged in the top bit),
          // written where they are read: every entry of a row the bitmap kernel
          // walks (zero for the other kinds), and every galloping entry
          uint2 sl = make_uint2(0u, 0u);
          if (kind == ACCX_KIND_BITMAP || kind == ACCX_KIND_GALLOP) {
            const uint32_t sst = ss[j];
            uint32_t tt = sst + dv;
            if (v > u) {  // cut P(v) at u: u's position in N(v) is the reverse entry
              const uint32_t r = __ldg(rev + e);
              tt = (r >= sst && r < tt) ? r : sst;
            }
            sl = make_uint2(sst, (tt - sst) | (kind == ACCX_KIND_GALLOP ? OR_SL_GALLOP : 0u));
            bwork = tt - sst;
          }
          if ((u < bm_idlim && du <= bm_pcap) || kind == ACCX_KIND_GALLOP) or_sl[e] = sl;
        }
        st.add(kind, dv, du);
        cm += kind == ACCX_KIND_MERGE;
        cg += kind == ACCX_KIND_GALLOP;
        if (kind == ACCX_KIND_BITMAP) {
          if (u != run_u) {
            if (run_u != 0xffffffffu) atomicAdd(&work_u[run_u], run_w + 1ull);
            run_u = u;
            run_w = 0;
          }
          run_w += bwork;
        }
        kinds |= (uint32_t)(kind < 0 || kind >= ACCX_NUM_KINDS ? 0xf : kind) << (4 * j);
      }
    }
    // the last run of every thread: lanes of one row add up first (long rows span
    // many threads)
    {
      const unsigned peers = __match_any_sync(ACCX_FULL_MASK, run_u);
      const unsigned long long hi = __reduce_add_sync(peers, (unsigned)(run_w >> 32));
      const unsigned long long lo = __reduce_add_sync(peers, (unsigned)(run_w & 0xffffffffu));
      if (run_u != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&work_u[run_u], (hi << 32) + lo + 1ull);
    }
    // list slots: exclusive scan of the threads' counts over the block
    uint32_t im = cm, ig = cg;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t a = __shfl_up_sync(ACCX_FULL_MASK, im, d), b = __shfl_up_sync(ACCX_FULL_MASK, ig, d);
      if (lane >= d) {
        im += a;
        ig += b;
      }
    }
    if (lane == 31) {
      s_wc[0][warp] = im;
      s_wc[1][warp] = ig;
    }
    __syncthreads();
    if (tid < 2) {
      uint32_t tot = 0;
      for (int w = 0; w < 8; w++) {
        const uint32_t c = s_wc[tid][w];
        s_wc[tid][w] = tot;
        tot += c;
      }
      s_base[tid] = tot ? atomicAdd(&ctr[tid == 0 ? C_MERGE : C_GALLOP], (unsigned long long)tot) : 0ull;
    }
    __syncthreads();
    if (cm | cg) {
      unsigned long long pm = s_base[0] + s_wc[0][warp] + im - cm, pg = s_base[1] + s_wc[1][warp] + ig - cg;
#pragma unroll
      for (int j = 0; j < CL_EPT; j++) {
        const uint32_t k = (kinds >> (4 * j)) & 0xfu;
        // owned edges number exactly m/2 on a symmetric graph; the guard only
        // keeps unvalidated asymmetric input inside the list
        if (k == ACCX_KIND_MERGE) {
          if (pm < list_cap) list[pm] = make_uint2(uu[j], e0 + (uint32_t)j);
          pm++;
        } else if (k == ACCX_KIND_GALLOP) {
          if (pg < list_cap) list[list_cap - 1 - pg] = make_uint2(uu[j], e0 + (uint32_t)j);
          pg++;
        }
      }
    }
    __syncthreads();  // s_wc and s_base are rewritten by the next block
  }
  // the statistics: warp sums, then the CTA's, then the device counters
  static_assert(C_WORK == C_EDGES + ACCX_NUM_KINDS && C_OWNER == C_WORK + ACCX_NUM_KINDS, "counter layout");
#pragma unroll
  for (int k = 0; k < ACCX_NUM_KINDS; k++) {
    unsigned long long v3[3] = {st.e[k], st.w[k], st.o[k]};
#pragma unroll
    for (int q = 0; q < 3; q++) {
      unsigned long long x = v3[q];
#pragma unroll
      for (int d = 16; d >= 1; d >>= 1) x += __shfl_xor_sync(ACCX_FULL_MASK, x, d);
      if (lane == 0 && x) atomicAdd(&s_st[q * ACCX_NUM_KINDS + k], x);
    }
  }
  __syncthreads();
  if (tid < 3 * ACCX_NUM_KINDS && s_st[tid]) atomicAdd(&ctr[C_EDGES + tid], s_st[tid]);
}

// ---------------------------------------------------------------------------
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
// Bitmap work items.  A bitmap owner u (an owner with at least one bitmap-kind
// edge) stages N(u) in shared memory as two parts: ids below W in a dense
// bitmap (after the degree-descending relabel these are the highest-degree
// vertices, where most probes land), ids from W up as (word index -> 32-bit
// word) pairs in an open-addressing table.  If the upper part has more ids than
// half the table's slots it is cut into chunks; the owner then becomes
// nchunks x nsplit virtual items (chunk c, split s probes the owned entries in
// the s-th slice of N(u)).  Only per-owner item counts are stored; a CTA maps an
// item index to its owner by a warp-parallel search over their prefix.
__device__ __forceinline__ void accx_item_shape(uint32_t du, uint32_t nsp, unsigned long long work, uint32_t chs,
                                                uint32_t target, uint32_t *nchunks, uint32_t *nsplit) {
  uint32_t nc = (nsp + chs - 1) / chs;
  if (nc < 1) nc = 1;
  unsigned long long per = (unsigned long long)nc * target;
  unsigned long long ns = (work + per - 1) / per;
  unsigned long long nsmax = du / 32 > 1 ? du / 32 : 1;
  if (ns > nsmax) ns = nsmax;
  if (ns < 1) ns = 1;
  *nchunks = nc;
  *nsplit = (uint32_t)ns;
}

__global__ void k_item_counts(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst, uint32_t n,
                              const unsigned long long *__restrict__ work_u, uint32_t W, uint32_t chs,
                              uint32_t target, unsigned long long *__restrict__ icnt,
                              unsigned long long *__restrict__ ctr, const uint32_t *__restrict__ pre) {
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u <= n; u += gridDim.x * blockDim.x) {
    unsigned long long c = 0;
    if (u < n) {
      unsigned long long w = work_u[u];
      if (w) {
        uint32_t ub = off[u], ue = off[u + 1];
        // oriented owners stage only their prefix, all of it in the dense window
        uint32_t us = pre ? ue : accx_lower_bound(dst, ub, ue, (int32_t)min(W, 0x7fffffffu));
        uint32_t nc, ns;
        accx_item_shape(ue - ub, ue - us, w, chs, target, &nc, &ns);
        c = (unsigned long long)nc * ns;
        atomicAdd(&ctr[C_OWNER + ACCX_KIND_BITMAP], (unsigned long long)(pre ? pre[u] : ue - ub) * ns);
      }
    }
    icnt[u] = c;
  }
}

__device__ __forceinline__ uint32_t accx_slot_hash(uint32_t word, uint32_t S) {
  return __umulhi(word * 0x9E3779B1u, S);
}

__device__ __forceinline__ void accx_sparse_insert(uint2 *slots, uint32_t S, uint32_t x) {
  const uint32_t key = (x >> 5) + 1u;
  uint32_t h = accx_slot_hash(x >> 5, S);
  for (uint32_t it = 0; it < S; it++) {
    uint32_t prev = atomicCAS(&slots[h].x, 0u, key);
    if (prev == 0u || prev == key) {
      atomicOr(&slots[h].y, 1u << (x & 31));
      return;
    }
    h = (h + 1 == S) ? 0 : h + 1;
  }
}

__device__ __forceinline__ uint32_t accx_sparse_find(const uint2 *slots, uint32_t S, uint32_t x, bool *hit) {
  const uint32_t key = (x >> 5) + 1u;
  uint32_t h = accx_slot_hash(x >> 5, S);
  for (uint32_t it = 0; it < S; it++) {
    uint2 s = slots[h];
    if (s.x == key) {
      *hit = (s.y >> (x & 31)) & 1u;
      return h;
    }
    if (s.x == 0u) break;
    h = (h + 1 == S) ? 0 : h + 1;
  }
  *hit = false;
  return 0xffffffffu;
}

struct accx_bm_view {
  const uint32_t *words;
  const uint2 *slots;
  uint32_t W, S;
  bool has_sparse;
};

__device__ __forceinline__ uint32_t accx_bm_test(const accx_bm_view &b, uint32_t x) {
  if (x < b.W) return (b.words[x >> 5] >> (x & 31)) & 1u;
  if (!b.has_sparse) return 0u;
  bool hit;
  accx_sparse_find(b.slots, b.S, x, &hit);
  return hit ? 1u : 0u;
}

#define PROBE_UNROLL 4  // ids per lane in a chunk of concatenated short lists
// probe lists of at least LONG_SEG ids go whole to one warp, shorter ones are
// concatenated; at R-MAT scale 24 the oriented kernel measured 32: +2.3%, 48: +0.7%, 128: +2.2%
#define LONG_SEG 64
#ifndef GALLOP_OR_GROUP
#define GALLOP_OR_GROUP 8  // lanes per galloping edge in oriented counts (16: +24%, 32: +70% galloping time)
#endif

// One CTA per virtual item (grid-stride).  Per round of up to blockDim owned
// entries, each thread takes one entry (u,v) and the part of N(v) to probe.
// Long parts (>= LONG_SEG ids) are pulled by whole warps and streamed with
// 16-byte loads; short parts are concatenated (CTA prefix sum) and streamed 32
// ids per warp step, a lane finding its entry from a ballot-built boundary mask.
// Hits are counted per entry (registers for long parts, shared counters for
// short ones).
__global__ void __launch_bounds__(1024, 1) k_bitmap(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                                    uint32_t n, int policy, const uint8_t *__restrict__ table,
                                                    const unsigned long long *__restrict__ work_u,
                                                    const unsigned long long *__restrict__ prefix, uint32_t W,
                                                    uint32_t S, uint32_t target, int32_t *__restrict__ cnt) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t *words = smem;                                   // W/32 dense words
  uint2 *slots = reinterpret_cast<uint2 *>(smem + W / 32);  // S sparse slots
  __shared__ uint8_t s_table[ACCX_NB * ACCX_NB];
  __shared__ uint32_t s_u, s_us, s_tot, s_nseg, s_nlong, s_lnext;
  __shared__ uint32_t s_wsum[32], s_wcnt[32], s_wlong[32];
  __shared__ uint32_t s_pre[1025], s_beg[1024], s_ent[1024], s_hit[1024];
  __shared__ uint32_t s_lbeg[1024], s_llen[1024], s_lent[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const uint32_t CHS = S / 2;
  const uint32_t nwords = W / 32;
  for (int i = tid; i < ACCX_NB * ACCX_NB; i += nt) s_table[i] = table ? table[i] : 0;
  for (uint32_t i = tid; i < nwords; i += nt) words[i] = 0;
  for (uint32_t i = tid; i < S; i += nt) slots[i] = make_uint2(0u, 0u);
  const unsigned long long total = prefix[n];
  __syncthreads();
  for (unsigned long long it = blockIdx.x; it < total; it += gridDim.x) {
    if (warp == 0) {
      // largest u in [0, n) with prefix[u] <= it (that owner has >= 1 item)
      uint32_t lo = 0, hi = n;
      while (hi - lo > 1) {
        uint32_t step = (hi - lo + 31) / 32;
        uint32_t p = lo + (uint32_t)lane * step;
        bool ok = p < hi && prefix[p] <= it;
        unsigned b = __ballot_sync(ACCX_FULL_MASK, ok);
        lo = lo + (31 - __clz(b)) * step;
        uint32_t nh = lo + step;
        hi = nh < hi ? nh : hi;
      }
      if (lane == 0) {
        s_u = lo;
        s_us = accx_lower_bound(dst, off[lo], off[lo + 1], (int32_t)min(W, 0x7fffffffu));
      }
    }
    __syncthreads();
    const uint32_t u = s_u, us = s_us;
    const uint32_t ub = off[u], ue = off[u + 1], du = ue - ub;
    uint32_t nchunks, nsplit;
    accx_item_shape(du, ue - us, work_u[u], CHS, target, &nchunks, &nsplit);
    const uint32_t j = (uint32_t)(it - prefix[u]);
    const uint32_t c = j / nsplit, sp = j % nsplit;
    const uint32_t ca = min(ue, us + c * CHS), cb = min(ue, ca + CHS);
    const uint32_t pa = ub + (uint32_t)((unsigned long long)du * sp / nsplit);
    const uint32_t pb = ub + (uint32_t)((unsigned long long)du * (sp + 1) / nsplit);
    const bool windowed = nchunks > 1;
    const bool dense_part = (c == 0) && us > ub;
    accx_bm_view bv{words, slots, W, S, cb > ca};
    const int32_t u_lo = __ldg(dst + ub), u_hi = __ldg(dst + ue - 1);
    const int32_t c_lo = cb > ca ? __ldg(dst + ca) : 0, c_hi = cb > ca ? __ldg(dst + cb - 1) : 0;
    // stage
    if (dense_part)
      for (uint32_t i = ub + tid; i < us; i += nt) {
        uint32_t x = (uint32_t)__ldg(dst + i);
        if (x < W) atomicOr(&words[x >> 5], 1u << (x & 31));
      }
    for (uint32_t i = ca + tid; i < cb; i += nt) accx_sparse_insert(slots, S, (uint32_t)__ldg(dst + i));
    __syncthreads();
    // probe, one round of up to nt owned entries at a time
    for (uint32_t r0 = pa; r0 < pb; r0 += (uint32_t)nt) {
      const uint32_t k = r0 + (uint32_t)tid;
      uint32_t sst = 0, len = 0;
      if (k < pb) {
        const uint32_t v = (uint32_t)__ldg(dst + k);
        const uint32_t vb = __ldg(off + v), ve = __ldg(off + v + 1), dv = ve - vb;
        if (dv > 0 && accx_owns(u, du, v, dv) &&
            accx_edge_kind(policy, s_table, du, dv) == ACCX_KIND_BITMAP) {
          uint32_t t = ve;
          sst = vb;
          if (!windowed) {
            if (__ldg(dst + ve - 1) < u_lo || __ldg(dst + vb) > u_hi) t = sst;  // disjoint id spans
          } else {
            if (c > 0) sst = accx_lower_bound(dst, vb, ve, c_lo);
            t = accx_lower_bound(dst, sst, ve, c_hi + 1);
          }
          len = t - sst;  // an empty part leaves the zeroed count in place
        }
      }
      // compact: short parts (prefix-summed) and long parts (a work list)
      const bool is_short = len > 0 && len < LONG_SEG, is_long = len >= LONG_SEG;
      const unsigned bs = __ballot_sync(ACCX_FULL_MASK, is_short), bl = __ballot_sync(ACCX_FULL_MASK, is_long);
      const uint32_t slen = is_short ? len : 0u;
      uint32_t incl = slen;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(ACCX_FULL_MASK, incl, d);
        if (lane >= d) incl += y;
      }
      if (lane == 31) {
        s_wsum[warp] = incl;
        s_wcnt[warp] = __popc(bs);
        s_wlong[warp] = __popc(bl);
      }
      __syncthreads();
      if (warp == 0) {
        uint32_t ws = lane < nwarps ? s_wsum[lane] : 0u, wc = lane < nwarps ? s_wcnt[lane] : 0u;
        uint32_t wl = lane < nwarps ? s_wlong[lane] : 0u;
        uint32_t is = ws, ic = wc, il = wl;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          uint32_t y = __shfl_up_sync(ACCX_FULL_MASK, is, d), z = __shfl_up_sync(ACCX_FULL_MASK, ic, d);
          uint32_t q = __shfl_up_sync(ACCX_FULL_MASK, il, d);
          if (lane >= d) { is += y; ic += z; il += q; }
        }
        if (lane < nwarps) { s_wsum[lane] = is - ws; s_wcnt[lane] = ic - wc; s_wlong[lane] = il - wl; }
        if (lane == 31) { s_tot = is; s_nseg = ic; s_nlong = il; s_lnext = 0; }
      }
      __syncthreads();
      if (is_short) {
        const uint32_t idx = s_wcnt[warp] + __popc(bs & ((1u << lane) - 1u));
        s_pre[idx] = s_wsum[warp] + incl - len;
        s_beg[idx] = sst;
        s_ent[idx] = k;
        s_hit[idx] = 0;
      }
      if (is_long) {
        const uint32_t idx = s_wlong[warp] + __popc(bl & ((1u << lane) - 1u));
        s_lbeg[idx] = sst;
        s_llen[idx] = len;
        s_lent[idx] = k;
      }
      __syncthreads();
      const uint32_t tot = s_tot, nseg = s_nseg, nlong = s_nlong;
      if (tid == 0) s_pre[nseg] = tot;
      __syncthreads();
      // short parts: each warp takes 32*PROBE_UNROLL consecutive ids of the concatenation
      for (uint32_t c0 = (uint32_t)warp * 32u * PROBE_UNROLL; c0 < tot; c0 += (uint32_t)nwarps * 32u * PROBE_UNROLL) {
        uint32_t lo = 0, hi = nseg;
        while (hi - lo > 1) {
          uint32_t step = (hi - lo + 31) / 32;
          uint32_t p = lo + (uint32_t)lane * step;
          unsigned b = __ballot_sync(ACCX_FULL_MASK, p < hi && s_pre[p] <= c0);
          lo += (31 - __clz(b)) * step;
          uint32_t nh = lo + step;
          hi = nh < hi ? nh : hi;
        }
        // segb = part holding the sub-chunk's first id; 32 ids meet at most 31
        // part starts after it, so each lane loads one start, the warp ORs them
        // into a mask by offset, and a lane's part is segb + (starts at or before it).
        uint32_t segb = lo;
        int32_t xs[PROBE_UNROLL];
        uint32_t sg[PROBE_UNROLL];
#pragma unroll
        for (int r = 0; r < PROBE_UNROLL; r++) {
          const uint32_t i0 = c0 + 32u * r;
          const uint32_t i = i0 + (uint32_t)lane;
          const uint32_t kb = segb + 1u + (uint32_t)lane;
          const uint32_t bnd = kb <= nseg ? s_pre[kb] : 0xffffffffu;
          const uint32_t o = bnd - i0;  // >= 1: part segb holds i0
          const unsigned M = __reduce_or_sync(ACCX_FULL_MASK, o < 32u ? (1u << o) : 0u);
          const uint32_t sj = segb + __popc(M & (lane == 31 ? 0xffffffffu : ((2u << lane) - 1u)));
          sg[r] = sj;
          xs[r] = (i < tot) ? __ldg(dst + s_beg[sj] + (i - s_pre[sj])) : -1;
          segb += __popc(M) + (__ballot_sync(ACCX_FULL_MASK, o == 32u) ? 1u : 0u);
        }
#pragma unroll
        for (int r = 0; r < PROBE_UNROLL; r++)
          if (xs[r] >= 0 && accx_bm_test(bv, (uint32_t)xs[r])) atomicAdd(&s_hit[sg[r]], 1u);
      }
      // long parts: whole warps, 16-byte loads
      for (;;) {
        uint32_t q = 0;
        if (lane == 0) q = atomicAdd(&s_lnext, 1u);
        q = __shfl_sync(ACCX_FULL_MASK, q, 0);
        if (q >= nlong) break;
        const uint32_t a0 = s_lbeg[q], a1 = a0 + s_llen[q];
        const uint32_t al = min(a1, (a0 + 3u) & ~3u), bl4 = max(al, a1 & ~3u);
        uint32_t h = 0;
        if (a0 + (uint32_t)lane < al) h += accx_bm_test(bv, (uint32_t)__ldg(dst + a0 + lane));
        if (bl4 + (uint32_t)lane < a1) h += accx_bm_test(bv, (uint32_t)__ldg(dst + bl4 + lane));
        for (uint32_t jj = al + 4u * (uint32_t)lane; jj < bl4; jj += 256u) {
          const int4 q0 = __ldg(reinterpret_cast<const int4 *>(dst + jj));
          int4 q1 = make_int4(-1, -1, -1, -1);
          if (jj + 128u < bl4) q1 = __ldg(reinterpret_cast<const int4 *>(dst + jj + 128u));
          h += accx_bm_test(bv, (uint32_t)q0.x) + accx_bm_test(bv, (uint32_t)q0.y) +
               accx_bm_test(bv, (uint32_t)q0.z) + accx_bm_test(bv, (uint32_t)q0.w);
          if (q1.x >= 0)
            h += accx_bm_test(bv, (uint32_t)q1.x) + accx_bm_test(bv, (uint32_t)q1.y) +
                 accx_bm_test(bv, (uint32_t)q1.z) + accx_bm_test(bv, (uint32_t)q1.w);
        }
        h = __reduce_add_sync(ACCX_FULL_MASK, h);
        if (lane == 0) {
          const uint32_t kk = s_lent[q];
          if (windowed) {
            if (h) atomicAdd(&cnt[kk], (int32_t)h);
          } else {
            cnt[kk] = (int32_t)h;
          }
        }
      }
      __syncthreads();
      for (uint32_t q = tid; q < nseg; q += nt) {
        const uint32_t h = s_hit[q], kk = s_ent[q];
        if (windowed) {
          if (h) atomicAdd(&cnt[kk], (int32_t)h);
        } else {
          cnt[kk] = (int32_t)h;
        }
      }
      __syncthreads();
    }
    // clear what was staged
    if (dense_part) {
      if ((us - ub) * 8u > nwords) {
        for (uint32_t i = tid; i < nwords; i += nt) words[i] = 0;
      } else {
        for (uint32_t i = ub + tid; i < us; i += nt) {
          uint32_t x = (uint32_t)__ldg(dst + i);
          if (x < W) words[x >> 5] = 0;
        }
      }
    }
    const uint32_t nel = cb - ca;
    if (nel && nel <= 4u * (uint32_t)nt) {
      uint32_t hs[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        uint32_t i = ca + tid + (uint32_t)r * nt;
        bool dummy;
        hs[r] = i < cb ? accx_sparse_find(slots, S, (uint32_t)__ldg(dst + i), &dummy) : 0xffffffffu;
      }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < 4; r++)
        if (hs[r] != 0xffffffffu) slots[hs[r]] = make_uint2(0u, 0u);
    } else if (nel) {
      for (uint32_t i = tid; i < S; i += nt) slots[i] = make_uint2(0u, 0u);
    }
    __syncthreads();
  }
}

#include "orient.cuh"

// ---------------------------------------------------------------------------
// Mirror: each owned entry e=(u,v) adds the bias and copies its count to the
// reverse entry (the position of u in N(v)).
template <int TILE>
__global__ void __launch_bounds__(TILE) k_mirror(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow, const int32_t *__restrict__ dst,
                                                 uint32_t n, uint32_t m, int32_t bias, int32_t *__restrict__ cnt) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, tilerow, n, m, base, e, &sh);
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
  cudaStream_t h = g->home;
  if (!g->d_cnt) ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_cnt, sizeof(int32_t) * (m ? m : 1), h));
  if (!g->d_edge_list) ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_edge_list, sizeof(uint2) * (m / 2 + 1), h));
  if (!g->d_icnt) {
    ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_icnt, sizeof(unsigned long long) * (n + 1), h));
    ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_prefix, sizeof(unsigned long long) * (n + 1), h));
    ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_pre, sizeof(uint32_t) * (n ? n : 1), h));
    size_t bytes = 0;
    ACCX_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, bytes, g->d_icnt, g->d_prefix, (int64_t)n + 1));
    ACCX_CUDA_TRY(accx_dev_alloc(&g->d_scan_tmp, bytes ? bytes : 16, h));
    g->scan_tmp_bytes = bytes;
  }
  if (!g->d_counters) {
    // counters followed by the per-vertex bitmap work array
    ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_counters, sizeof(unsigned long long) * (C_NUM + n + 1), h));
  }
  if (!g->d_table) {
    ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_table, ACCX_NB * ACCX_NB, h));
    // pool allocations are ordered on the home stream; counts may run on another
    if (h) ACCX_CUDA_TRY(cudaStreamSynchronize(h));
  }
  return ACCX_OK;
}

int accx_prefix_lengths(accx_graph *g, cudaStream_t s) {
  int rc = accx_ensure_count_scratch(g);
  if (rc) return rc;
  const bool rel = g->d_roff != nullptr;
  if (g->n) k_pre<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(rel ? g->d_roff : g->d_off, rel ? g->d_rdst : g->d_dst,
                                                                g->n, g->d_pre, nullptr);
  ACCX_CUDA_TRY(cudaGetLastError());
  return ACCX_OK;
}

// Tuned defaults (overridable per call).  Oriented counts read bitmap_window_kb
// as the dense window and sparse_table_kb as the owner-prefix counters.
static int g_block_warps = 32;
static int g_dense_kb = 128;
static int g_sparse_kb = 64;
// Oriented bitmap kind: 256-thread CTAs, four per SM, with a 24 KiB window (owners
// with ids below 196,608 use the bitmap kind, the others gallop).  Small CTAs run
// a round's scans and barriers with fewer idle threads (most owners' rows are far
// shorter than a CTA), and the low-degree owners past the window are cheaper to
// gallop than to stage.  Whole counts (ms) by (CTA threads, window KiB):
//   R-MAT 22: 256/24 18.9, 512/56 24.1 (the earlier default), 256/16 18.4
//   R-MAT 24: 256/24 96.7, 512/56 98.6, 256/16 110.9 (too many owners gallop)
//   Chung-Lu 20M (exponent 2.1): 256/24 46.0, 512/56 ~49; Erdos-Renyi 20M: 32.1, ~33.3
// and with 256 threads a 32 KiB window (three CTAs per SM) or 128-thread CTAs
// were slower at R-MAT 24 (95.4 and 93.5-127.4 ms for the bitmap phase alone).
static int g_or_dense_kb = 24;
static int g_or_counter_kb = 8;
static int g_or_block_warps = 8;


// Persistent classify CTAs: four per SM (64 registers a thread), at most one per
// block of entries.
static unsigned classify_grid(int sms, uint32_t m) {
  const unsigned long long blocks = ((unsigned long long)m + 256 * CL_EPT - 1) / (256 * CL_EPT);
  const unsigned long long g = (unsigned long long)sms * 4;
  return (unsigned)(blocks < g ? (blocks ? blocks : 1) : g);
}

// host_out (optional): the caller's output as a device-mapped pointer; a count
// on the relabeled CSR then writes it in its final gather (*host_done = true).
static int launch_count(accx_graph *g, const accx_count_opts *o, cudaStream_t s, int32_t *host_out = nullptr,
                        bool *host_done = nullptr) {
  const uint32_t n = g->n, m = (uint32_t)g->m;
  int policy = o ? o->policy : ACCX_POLICY_HEURISTIC;
  int32_t bias = o ? o->bias : 0;
  const bool orient = o && o->orient;
  int warps = (o && o->block_warps > 0) ? o->block_warps : (orient ? g_or_block_warps : g_block_warps);
  int dkb = (o && o->bitmap_window_kb > 0) ? o->bitmap_window_kb : (orient ? g_or_dense_kb : g_dense_kb);
  int skb = (o && o->sparse_table_kb > 0) ? o->sparse_table_kb : (orient ? g_or_counter_kb : g_sparse_kb);
  if (policy < ACCX_POLICY_HEURISTIC || policy > ACCX_POLICY_MODEL) return ACCX_ERR_INVALID_ARG;
  if (o && (o->orient < 0 || o->orient > 1)) return ACCX_ERR_INVALID_ARG;
  if (warps < 1 || warps > 32 || dkb < 1 || skb < 1) return ACCX_ERR_INVALID_ARG;
  if (orient ? (dkb + dkb / 2 + skb > 196 || skb > 200) : (dkb + skb > 200)) return ACCX_ERR_INVALID_ARG;
  if (n == 0) {
    g->cnt_bias = bias;
    g->cnt_valid = true;
    return ACCX_OK;
  }
  int rc = accx_ensure_count_scratch(g);
  if (rc) return rc;
  if (policy == ACCX_POLICY_TABLE) {
    if (!o->table) return ACCX_ERR_INVALID_ARG;
    for (int i = 0; i < ACCX_NB * ACCX_NB; i++)
      if (o->table[i] > ACCX_KIND_SKIP) return ACCX_ERR_INVALID_ARG;
    ACCX_CUDA_TRY(cudaMemcpyAsync(g->d_table, o->table, ACCX_NB * ACCX_NB, cudaMemcpyHostToDevice, s));
    ACCX_CUDA_TRY(cudaStreamSynchronize(s));  // o->table is pageable caller memory
  } else if (policy == ACCX_POLICY_MODEL) {
    rc = accx_model_table_device(g, s, orient ? 1 : 0);  // the attached model writes g->d_table on the device
    if (rc) return rc;
  }
  // counting runs on the relabeled CSR when the handle has one
  const bool rel = g->d_roff != nullptr;
  const uint32_t *off = rel ? g->d_roff : g->d_off;
  const int32_t *dst = rel ? g->d_rdst : g->d_dst;
  int32_t *cnt = rel ? g->d_rcnt : g->d_cnt;
  if (!(rel ? g->d_rtilerow : g->d_tilerow)) {  // e.g. a graph built from an edge list
    rc = accx_tilerow_build(g, off, rel ? &g->d_rtilerow : &g->d_tilerow, s);
    if (rc) return rc;
  }
  const uint32_t *tilerow = rel ? g->d_rtilerow : g->d_tilerow;
  unsigned long long *ctr = g->d_counters;
  unsigned long long *work_u = g->d_counters + C_NUM;
  ACCX_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long) * (C_NUM + (size_t)n + 1), s));
  if (!orient) ACCX_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)(m ? m : 1), s));
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
  int sms = accx_sm_count(g->device);
  if (o && o->sm_limit > 0 && o->sm_limit < sms) sms = o->sm_limit;
  if (orient) {
    const uint32_t W = (uint32_t)dkb * 8192u;       // dense ids (bits); bitmap owners have ids below W
    const uint32_t pcap = (uint32_t)skb * 256u;     // owner-prefix counters
    // words + the zero word (padded), owner counters + 32 spares, word ranks
    const size_t smem = (size_t)W / 8u + 16u + ((size_t)pcap + 32u) * 4u + (size_t)W / 16u;
    const uint32_t target = ITEM_TARGET_DEFAULT;
    // per-entry bitmap work and the item array (n + m/32 + 1 bounds the items:
    // an owner is cut into at most max(1, degree/32) slices)
    const uint32_t items_cap = n + m / 32u + 1u;
    if (!g->d_or_sl || !g->d_or_items || !g->d_vinfo) {
      if (!g->d_or_sl) ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_or_sl, sizeof(uint2) * (size_t)m, g->home));
      if (!g->d_vinfo) ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_vinfo, sizeof(uint2) * (size_t)n, g->home));
      if (!g->d_or_items)
        ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_or_items, sizeof(uint32_t) * (size_t)items_cap, g->home));
      if (g->home) ACCX_CUDA_TRY(cudaStreamSynchronize(g->home));
    }
    k_pre<<<sms * 8, 256, 0, s>>>(off, dst, n, g->d_pre, g->d_vinfo);
    // reverse entries: built on the first oriented count of this CSR and kept
    // (an index of the graph, like the tile rows).  The original CSR's comes
    // from validation; a known-symmetric CSR's from the sort (accx_rev_by_sort);
    // otherwise, or when the sort's scratch does not fit, a search per entry
    // pair, which leaves 0xffffffff where an asymmetric CSR has no reverse.
    if (g->rev_csr != off) {
      uint32_t *sorted = nullptr;
      if (g->d_rev_orig && !rel) {  // recorded by validation for this very CSR
        std::swap(g->d_rev, g->d_rev_orig);
        accx_dev_free(g->d_rev_orig, g->home);
        g->d_rev_orig = nullptr;
      } else {
        rc = g->symmetric ? accx_rev_by_sort(g, off, tilerow, dst, nullptr, s, &sorted) : ACCX_ERR_OOM;
        if (rc == ACCX_OK) {
          accx_dev_free(g->d_rev, g->home);
          g->d_rev = sorted;
        } else if (rc == ACCX_ERR_OOM) {
          if (!g->d_rev) {
            ACCX_CUDA_TRY(accx_dev_alloc((void **)&g->d_rev, sizeof(uint32_t) * (size_t)m, g->home));
            if (g->home) ACCX_CUDA_TRY(cudaStreamSynchronize(g->home));
          }
          ACCX_CUDA_TRY(cudaMemsetAsync(g->d_rev, 0xff, sizeof(uint32_t) * (size_t)m, s));
          k_rev_build<256><<<tiles, 256, 0, s>>>(off, tilerow, dst, g->d_pre, n, m, g->d_rev);
        } else {
          return rc;
        }
      }
      g->rev_csr = off;
    }
    k_classify<true><<<classify_grid(sms, m), 256, 0, s>>>(off, tilerow, dst, n, m, policy, g->d_table, g->d_edge_list,
                                                          list_cap, work_u, ctr, g->d_pre, W, pcap, g->d_or_sl, g->d_rev,
                                                          cnt, bias, g->d_vinfo);  // classify also fills cnt with the bias
    k_item_counts<<<sms * 4, 256, 0, s>>>(off, dst, n, work_u, W, 1, target, g->d_icnt, ctr, g->d_pre);
    ACCX_CUDA_TRY(cub::DeviceScan::ExclusiveSum(g->d_scan_tmp, g->scan_tmp_bytes, g->d_icnt, g->d_prefix,
                                                (int64_t)n + 1, s));
    k_item_fill<<<sms * 4, 256, 0, s>>>(g->d_icnt, g->d_prefix, n, items_cap, g->d_or_items);
    ACCX_MARK(1);
    k_merge_or<<<sms * 8, MERGE_WARPS * 32, 0, s>>>(off, dst, g->d_pre, g->d_rev, g->d_edge_list, list_cap, ctr,
                                                    cnt);
    ACCX_MARK(2);
    k_gallop_or<GALLOP_OR_GROUP><<<sms * 8, MERGE_WARPS * 32, 0, s>>>(g->d_vinfo, dst, g->d_or_sl, g->d_edge_list, list_cap, ctr,
                                                     cnt);
    ACCX_MARK(3);
    // the instance whose per-round arrays fit the block: 256 threads (four CTAs per
    // SM with the default 24 KiB window), 512 (two per SM with windows up to ~60
    // KiB) or 1024
    auto kb = warps <= 8 ? k_bitmap_or<256> : warps <= 16 ? k_bitmap_or<512> : k_bitmap_or<1024>;
    ACCX_CUDA_TRY(cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    ACCX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kb, warps * 32, smem));
    if (per_sm < 1) return ACCX_ERR_INVALID_ARG;
    kb<<<sms * per_sm, warps * 32, smem, s>>>(off, dst, g->d_pre, n, g->d_or_items, items_cap, work_u, g->d_prefix,
                                              g->d_or_sl, W, pcap, target, cnt, ctr);
    ACCX_MARK(4);
    // suffix entries take their prefix entry's count.  One thread per entry in
    // entry order, so the reads of the prefix entries sweep the array upwards;
    // reading them through a precomputed index in the caller's entry order
    // instead (and skipping this pass) was measured slower (R-MAT 24: 7.5 ms
    // against 5.1 ms for this pass and the gather).
    k_combine_or<<<tiles, 256, 0, s>>>(m, g->d_rev, cnt);
  } else {
    k_classify<false><<<classify_grid(sms, m), 256, 0, s>>>(off, tilerow, dst, n, m, policy, g->d_table, g->d_edge_list,
                                                           list_cap, work_u, ctr, nullptr, 0u, 0u, nullptr, nullptr,
                                                           nullptr, 0, nullptr);
    const uint32_t W = (uint32_t)dkb * 8192u;        // dense ids (bits)
    const uint32_t S = (uint32_t)skb * 1024u / 8u;   // sparse 8-byte slots
    const size_t smem = (size_t)W / 8u + (size_t)S * 8u;
    const uint32_t target = ITEM_TARGET_DEFAULT;
    k_item_counts<<<sms * 4, 256, 0, s>>>(off, dst, n, work_u, W, S / 2, target, g->d_icnt, ctr, nullptr);
    ACCX_CUDA_TRY(cub::DeviceScan::ExclusiveSum(g->d_scan_tmp, g->scan_tmp_bytes, g->d_icnt, g->d_prefix,
                                                (int64_t)n + 1, s));
    ACCX_MARK(1);
    k_merge<<<sms * 8, MERGE_WARPS * 32, 0, s>>>(off, dst, g->d_edge_list, list_cap, ctr, cnt);
    ACCX_MARK(2);
    k_gallop<<<sms * 8, MERGE_WARPS * 32, 0, s>>>(off, dst, g->d_edge_list, list_cap, ctr, cnt);
    ACCX_MARK(3);
    ACCX_CUDA_TRY(cudaFuncSetAttribute(k_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    ACCX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bitmap, warps * 32, smem));
    if (per_sm < 1) return ACCX_ERR_INVALID_ARG;
    k_bitmap<<<sms * per_sm, warps * 32, smem, s>>>(off, dst, n, policy, g->d_table, work_u, g->d_prefix, W, S, target,
                                                    cnt);
    ACCX_MARK(4);
    k_mirror<256><<<tiles, 256, 0, s>>>(off, tilerow, dst, n, m, bias, cnt);
  }
  if (rel) {
    rc = accx_relabel_gather(g, host_out, s);
    if (rc) return rc;
    if (host_out && host_done) *host_done = true;
  }
  ACCX_MARK(5);
#undef ACCX_MARK
  ACCX_CUDA_TRY(cudaGetLastError());
  g->cnt_bias = bias;
  g->cnt_valid = true;
  g->qc.query_valid = false;
  g->qc.pairs_valid = false;
  g->key_valid.store(false, std::memory_order_release);
  return ACCX_OK;
}

extern "C" int accx_cn_count(accx_graph *g, const accx_count_opts *opts, int32_t *out, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  ACCX_CUDA_TRY(cudaSetDevice(g->device));
  // pinned host output, 16-byte aligned: written by the count's last pass itself
  int32_t *mapped = out ? static_cast<int32_t *>(accx_mapped_host(out)) : nullptr;
  if (mapped && ((uintptr_t)mapped & 15)) mapped = nullptr;
  bool done = false;
  int rc = launch_count(g, opts, s, mapped, &done);
  if (rc) {
    g->cnt_valid = false;
    return rc;
  }
  if (out && done) {
    ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  } else if (out) {
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

extern "C" int accx_cn_last_matches(const accx_graph *g, uint64_t matches[ACCX_NUM_KINDS], uint64_t *probed) {
  if (!g || !g->d_counters) return ACCX_ERR_INVALID_ARG;
  unsigned long long h[C_NUM];
  ACCX_CUDA_TRY(cudaDeviceSynchronize());
  ACCX_CUDA_TRY(cudaMemcpy(h, g->d_counters, sizeof(h), cudaMemcpyDeviceToHost));
  for (int k = 0; k < ACCX_NUM_KINDS; k++)
    if (matches) matches[k] = h[C_MATCH + k];
  if (probed) *probed = h[C_PROBED];
  return ACCX_OK;
}

extern "C" int accx_cn_last_timings(const accx_graph *g, float ms[ACCX_NUM_PHASES]) {
  if (!g || !ms) return ACCX_ERR_INVALID_ARG;
  if (!g->timed || !g->ev[0]) return ACCX_ERR_NOT_READY;
  ACCX_CUDA_TRY(cudaEventSynchronize(g->ev[ACCX_NUM_PHASES]));
  for (int i = 0; i < ACCX_NUM_PHASES; i++) ACCX_CUDA_TRY(cudaEventElapsedTime(&ms[i], g->ev[i], g->ev[i + 1]));
  return ACCX_OK;
}

extern "C" int accx_cn_read(const accx_graph *g, int32_t *out, void *stream) {
  if (!g || (!out && g->m)) return ACCX_ERR_INVALID_ARG;
  if (!g->cnt_valid || !g->d_cnt) return ACCX_ERR_NOT_READY;
  return accx_copy_out(out, g->d_cnt, sizeof(int32_t) * (size_t)g->m, (cudaStream_t)stream);
}

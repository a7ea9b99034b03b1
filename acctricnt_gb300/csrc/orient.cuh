// Oriented all-edge counting: common-neighbour counts as triangle credits.
//
// |N(u) ∩ N(v)| for an edge (u,v) is the number of triangles through it.  With
// the prefix P(x) = N(x) ∩ [0, x) (the neighbours with smaller ids; after the
// degree-descending relabel the higher-degree ones, at most sqrt(2m) ids), every
// triangle a < b < c is met exactly once: on the edge (c,b), as the id a common
// to P(c) ∩ [0,b) and P(b).  Each meeting adds one to the three entries (c,b),
// (c,a) and (b,a); a final pass adds the two entries of every undirected edge
// and writes the sum (plus the bias) to both.  The per-edge kernels are those of
// the direct path with prefix lists: an owner (the endpoint with the longer
// prefix, ties: smaller id) and a partner, the probe side cut at the smaller id.
//
// Credits are fire-and-forget atomics (RED): the partner-side entry of a match
// is the entry being read, so a warp's credits land in the lines it just loaded.
// The bitmap kernel keeps the owner-side credits in shared counters (one per
// prefix entry, found as the word's base rank + a popcount) and adds them to
// HBM once per work item.
//
// Included by count.cu after the shared counting definitions.
#pragma once

#define LONG_UNROLL 8  // loads in flight per lane on long probe lists

// pre[u] = |N(u) ∩ [0, u)|.
__global__ void k_pre(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst, uint32_t n,
                      uint32_t *__restrict__ pre) {
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const uint32_t b = __ldg(off + u), e = __ldg(off + u + 1);
    pre[u] = accx_lower_bound(dst, b, e, (int32_t)u) - b;
  }
}

// The two prefix ranges of an owned edge (x owner, y = dst[e]), each cut at
// min(x, y): ids from there up cannot be common to both prefixes.
__device__ __forceinline__ void accx_or_ranges(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                               const uint32_t *__restrict__ pre, uint32_t x, uint32_t y,
                                               uint32_t *xb, uint32_t *xe, uint32_t *yb, uint32_t *ye) {
  *xb = __ldg(off + x);
  *xe = *xb + __ldg(pre + x);
  *yb = __ldg(off + y);
  *ye = *yb + __ldg(pre + y);
  if (y < x) *xe = accx_lower_bound(dst, *xb, *xe, (int32_t)y);
  else *ye = accx_lower_bound(dst, *yb, *ye, (int32_t)x);
}

__global__ void __launch_bounds__(MERGE_WARPS * 32) k_merge_or(const uint32_t *__restrict__ off,
                                                                const int32_t *__restrict__ dst,
                                                                const uint32_t *__restrict__ pre,
                                                                const uint2 *__restrict__ list, uint32_t list_cap,
                                                                unsigned long long *__restrict__ ctr,
                                                                int32_t *__restrict__ cnt) {
  __shared__ __align__(16) int32_t buf[MERGE_WARPS][2][MERGE_WIN];
  unsigned long long found = 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long total = ctr[C_MERGE];
  if (total > list_cap) total = list_cap;
  const unsigned long long nw = (unsigned long long)gridDim.x * MERGE_WARPS;
  for (unsigned long long it = (unsigned long long)blockIdx.x * MERGE_WARPS + w; it < total; it += nw) {
    const uint2 p = list[it];
    const uint32_t x = p.x, e = p.y, y = (uint32_t)__ldg(dst + e);
    uint32_t xb, xe, yb, ye;
    accx_or_ranges(off, dst, pre, x, y, &xb, &xe, &yb, &ye);
    const uint32_t c = accx_warp_merge_credit(dst, xb, xe, yb, ye, buf[w][0], buf[w][1], lane, cnt);
    if (lane == 0 && c) atomicAdd(cnt + e, (int32_t)c);
    found += c;
    __syncwarp();
  }
  if (lane == 0 && found) atomicAdd(&ctr[C_MATCH + ACCX_KIND_MERGE], found);
}

// Lanes take the partner's prefix ids in order and binary-search each in the
// owner's prefix; every round starts at the position the last lane reached.
__global__ void __launch_bounds__(MERGE_WARPS * 32) k_gallop_or(const uint32_t *__restrict__ off,
                                                                 const int32_t *__restrict__ dst,
                                                                 const uint32_t *__restrict__ pre,
                                                                 const uint2 *__restrict__ list, uint32_t list_cap,
                                                                 unsigned long long *__restrict__ ctr,
                                                                 int32_t *__restrict__ cnt) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long found = 0;
  unsigned long long total = ctr[C_GALLOP];
  if (total > list_cap) total = list_cap;
  const unsigned long long nw = (unsigned long long)gridDim.x * MERGE_WARPS;
  for (unsigned long long it = (unsigned long long)blockIdx.x * MERGE_WARPS + w; it < total; it += nw) {
    const uint2 p = list[list_cap - 1 - it];
    const uint32_t x = p.x, e = p.y, y = (uint32_t)__ldg(dst + e);
    uint32_t xb, xe, yb, ye;
    accx_or_ranges(off, dst, pre, x, y, &xb, &xe, &yb, &ye);
    uint32_t c = 0, lo = xb;
    for (uint32_t j0 = yb; j0 < ye && lo < xe; j0 += 32) {
      const uint32_t j = j0 + (uint32_t)lane;
      uint32_t pos = xe;
      if (j < ye) {
        const int32_t id = __ldg(dst + j);
        pos = accx_lower_bound(dst, lo, xe, id);
        if (pos < xe && __ldg(dst + pos) == id) {
          c++;
          atomicAdd(cnt + pos, 1);
          atomicAdd(cnt + j, 1);
        }
      }
      const uint32_t last_lane = (ye - j0 >= 32) ? 31u : (ye - j0 - 1);
      lo = __shfl_sync(ACCX_FULL_MASK, pos, (int)last_lane);
    }
    c = __reduce_add_sync(ACCX_FULL_MASK, c);
    if (lane == 0 && c) atomicAdd(cnt + e, (int32_t)c);
    found += c;
  }
  if (lane == 0 && found) atomicAdd(&ctr[C_MATCH + ACCX_KIND_GALLOP], found);
}

// Bitmap kind.  One CTA per work item (an owner x, or a slice of its list when
// the owner's probe work is large).  The owner's prefix -- ids below x, which
// the classifier keeps below W -- is staged as a dense bitmap over [0, W) plus,
// per non-empty 32-bit word, the prefix position of the word's first id (rank of
// an id = that base + popcount of the lower bits).  Then every owned entry
// (x,y) of the slice probes P(y) cut at min(x,y): short probe lists are
// concatenated across the CTA and streamed 32 ids per warp step, long ones are
// pulled by whole warps with 16-byte loads.  A hit at partner entry j credits
// cnt[j] (RED), the owner's shared counter of the id's rank, and the edge.
__global__ void __launch_bounds__(1024, 1) k_bitmap_or(const uint32_t *__restrict__ off,
                                                       const int32_t *__restrict__ dst,
                                                       const uint32_t *__restrict__ pre, uint32_t n, int policy,
                                                       const uint8_t *__restrict__ table,
                                                       const unsigned long long *__restrict__ work_u,
                                                       const unsigned long long *__restrict__ prefix, uint32_t W,
                                                       uint32_t pcap, uint32_t target, int32_t *__restrict__ cnt,
                                                       unsigned long long *__restrict__ ctr) {
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t nwords = W / 32;
  uint32_t *words = smem;                                          // nwords
  uint32_t *ocnt = smem + nwords;                                  // pcap owner-prefix counters
  uint16_t *wbase = reinterpret_cast<uint16_t *>(ocnt + pcap);     // nwords first-id positions
  __shared__ uint8_t s_table[ACCX_NB * ACCX_NB];
  __shared__ uint32_t s_u, s_tot, s_nseg, s_nlong, s_lnext;
  __shared__ uint32_t s_wsum[32], s_wcnt[32], s_wlong[32];
  __shared__ uint32_t s_pre[1025], s_beg[1024], s_ent[1024], s_hit[1024];
  __shared__ uint32_t s_lbeg[1024], s_llen[1024], s_lent[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  for (int i = tid; i < ACCX_NB * ACCX_NB; i += nt) s_table[i] = table ? table[i] : 0;
  for (uint32_t i = tid; i < nwords; i += nt) words[i] = 0;
  const unsigned long long total = prefix[n];
  unsigned long long found = 0, probed = 0;  // this thread's share, summed per warp at the end
  __syncthreads();
  for (unsigned long long it = blockIdx.x; it < total; it += gridDim.x) {
    if (warp == 0) {
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
      if (lane == 0) s_u = lo;
    }
    __syncthreads();
    const uint32_t x = s_u;
    const uint32_t ub = off[x], ue = off[x + 1], du = ue - ub, px = pre[x];
    uint32_t nchunks, nsplit;
    accx_item_shape(du, 0, work_u[x], 1, target, &nchunks, &nsplit);
    const uint32_t sp = (uint32_t)(it - prefix[x]);
    const uint32_t pa = ub + (uint32_t)((unsigned long long)du * sp / nsplit);
    const uint32_t pb = ub + (uint32_t)((unsigned long long)du * (sp + 1) / nsplit);
    const uint32_t pxs = px <= pcap ? px : 0;  // the classifier guarantees px <= pcap for bitmap owners
    // stage the prefix
    for (uint32_t i = tid; i < pxs; i += nt) {
      const uint32_t id = (uint32_t)__ldg(dst + ub + i);
      if (id < W) {
        atomicOr(&words[id >> 5], 1u << (id & 31));
        if (i == 0 || ((uint32_t)__ldg(dst + ub + i - 1) >> 5) != (id >> 5)) wbase[id >> 5] = (uint16_t)i;
      }
      ocnt[i] = 0;
    }
    __syncthreads();
    for (uint32_t r0 = pa; r0 < pb; r0 += (uint32_t)nt) {
      const uint32_t k = r0 + (uint32_t)tid;
      uint32_t sst = 0, len = 0;
      if (k < pb) {
        const uint32_t y = (uint32_t)__ldg(dst + k);
        const uint32_t py = __ldg(pre + y);
        if (py > 0 && accx_owns(x, px, y, py) && accx_edge_kind(policy, s_table, px, py) == ACCX_KIND_BITMAP) {
          sst = __ldg(off + y);
          uint32_t t = sst + py;
          if (y > x) t = accx_lower_bound(dst, sst, t, (int32_t)x);
          len = t - sst;
        }
      }
      const bool is_short = len > 0 && len < LONG_SEG, is_long = len >= LONG_SEG;
      const unsigned bs = __ballot_sync(ACCX_FULL_MASK, is_short), bl = __ballot_sync(ACCX_FULL_MASK, is_long);
      const uint32_t slen = is_short ? len : 0u;
      uint32_t incl = slen;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t v = __shfl_up_sync(ACCX_FULL_MASK, incl, d);
        if (lane >= d) incl += v;
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
          uint32_t a = __shfl_up_sync(ACCX_FULL_MASK, is, d), b = __shfl_up_sync(ACCX_FULL_MASK, ic, d);
          uint32_t q = __shfl_up_sync(ACCX_FULL_MASK, il, d);
          if (lane >= d) { is += a; ic += b; il += q; }
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
      probed += len;
      __syncthreads();
      // short parts
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
        uint32_t segb = lo;
        int32_t xs[PROBE_UNROLL];
        uint32_t sg[PROBE_UNROLL], gi[PROBE_UNROLL];
#pragma unroll
        for (int r = 0; r < PROBE_UNROLL; r++) {
          const uint32_t i0 = c0 + 32u * r;
          const uint32_t i = i0 + (uint32_t)lane;
          const uint32_t kb = segb + 1u + (uint32_t)lane;
          const uint32_t bnd = kb <= nseg ? s_pre[kb] : 0xffffffffu;
          const uint32_t o = bnd - i0;
          const unsigned M = __reduce_or_sync(ACCX_FULL_MASK, o < 32u ? (1u << o) : 0u);
          const uint32_t sj = segb + __popc(M & (lane == 31 ? 0xffffffffu : ((2u << lane) - 1u)));
          sg[r] = sj;
          gi[r] = (i < tot) ? s_beg[sj] + (i - s_pre[sj]) : 0u;
          xs[r] = (i < tot) ? __ldg(dst + gi[r]) : -1;
          segb += __popc(M) + (__ballot_sync(ACCX_FULL_MASK, o == 32u) ? 1u : 0u);
        }
#pragma unroll
        for (int r = 0; r < PROBE_UNROLL; r++) {
          const uint32_t id = (uint32_t)xs[r];
          if (xs[r] >= 0 && id < W) {
            const uint32_t wd = words[id >> 5], bit = 1u << (id & 31);
            if (wd & bit) {
              const uint32_t rk = wbase[id >> 5] + __popc(wd & (bit - 1u));
              atomicAdd(cnt + gi[r], 1);
              if (rk < pxs) atomicAdd(&ocnt[rk], 1u);  // always true on a sorted CSR
              atomicAdd(&s_hit[sg[r]], 1u);
            }
          }
        }
      }
      // long parts
      for (;;) {
        uint32_t q = 0;
        if (lane == 0) q = atomicAdd(&s_lnext, 1u);
        q = __shfl_sync(ACCX_FULL_MASK, q, 0);
        if (q >= nlong) break;
        const uint32_t a0 = s_lbeg[q], a1 = a0 + s_llen[q];
        uint32_t h = 0;
        // lane-consecutive ids, LONG_UNROLL loads in flight per lane: a warp's
        // credits for one load land in one 128-byte line of cnt
        for (uint32_t j0 = a0; j0 < a1; j0 += 32u * LONG_UNROLL) {
          int32_t v[LONG_UNROLL];
#pragma unroll
          for (int r = 0; r < LONG_UNROLL; r++) {
            const uint32_t j = j0 + 32u * r + (uint32_t)lane;
            v[r] = j < a1 ? __ldg(dst + j) : -1;
          }
#pragma unroll
          for (int r = 0; r < LONG_UNROLL; r++) {
            const uint32_t id = (uint32_t)v[r];
            if (v[r] >= 0 && id < W) {
              const uint32_t wd = words[id >> 5], bit = 1u << (id & 31);
              if (wd & bit) {
                const uint32_t rk = wbase[id >> 5] + __popc(wd & (bit - 1u));
                h++;
                atomicAdd(cnt + j0 + 32u * r + (uint32_t)lane, 1);
                if (rk < pxs) atomicAdd(&ocnt[rk], 1u);
              }
            }
          }
        }
        h = __reduce_add_sync(ACCX_FULL_MASK, h);
        if (lane == 0) found += h;
        if (lane == 0 && h) {
          const uint32_t kk = s_lent[q];
          if (kk - ub < pxs) atomicAdd(&ocnt[kk - ub], h);
          else atomicAdd(cnt + kk, (int32_t)h);
        }
      }
      __syncthreads();
      for (uint32_t q = tid; q < nseg; q += nt) {
        const uint32_t h = s_hit[q], kk = s_ent[q];
        found += h;
        if (h) {
          if (kk - ub < pxs) atomicAdd(&ocnt[kk - ub], h);
          else atomicAdd(cnt + kk, (int32_t)h);
        }
      }
      __syncthreads();
    }
    // owner-side credits to HBM, then clear what was staged
    for (uint32_t i = tid; i < pxs; i += nt) {
      const uint32_t h = ocnt[i];
      if (h) atomicAdd(cnt + ub + i, (int32_t)h);
    }
    const uint32_t span = min(nwords, x / 32u + 1u);
    if (span <= pxs) {
      for (uint32_t i = tid; i < span; i += nt) words[i] = 0;
    } else {
      for (uint32_t i = tid; i < pxs; i += nt) {
        const uint32_t id = (uint32_t)__ldg(dst + ub + i);
        if (id < W) words[id >> 5] = 0;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    found += __shfl_xor_sync(ACCX_FULL_MASK, found, d);
    probed += __shfl_xor_sync(ACCX_FULL_MASK, probed, d);
  }
  if (lane == 0) {
    if (found) atomicAdd(&ctr[C_MATCH + ACCX_KIND_BITMAP], found);
    if (probed) atomicAdd(&ctr[C_PROBED], probed);
  }
}

// Sum of the two entries of every undirected edge, plus the bias, into both.
// One thread per suffix entry e = (v,u), u > v; the other entry is v's position
// in u's prefix, a short list (at most sqrt(2m) ids after the degree relabel),
// where the reverse search from a prefix entry would walk a hub's long suffix.
template <int TILE>
__global__ void __launch_bounds__(TILE) k_combine_or(const uint32_t *__restrict__ off,
                                                     const uint32_t *__restrict__ tilerow,
                                                     const int32_t *__restrict__ dst,
                                                     const uint32_t *__restrict__ pre, uint32_t n, uint32_t m,
                                                     int32_t bias, int32_t *__restrict__ cnt) {
  __shared__ accx_tile_rows<TILE> sh;
  const uint32_t base = blockIdx.x * (uint32_t)TILE;
  const uint32_t e = base + threadIdx.x;
  const uint32_t v = accx_tile_row<TILE>(off, tilerow, n, m, base, e, &sh);
  if (e >= m) return;
  const uint32_t u = (uint32_t)dst[e];
  if (u <= v) return;
  const uint32_t ub = __ldg(off + u), ue = ub + __ldg(pre + u);
  const uint32_t r = accx_lower_bound(dst, ub, ue, (int32_t)v);
  int32_t c = cnt[e] + bias;
  if (r < ue && __ldg(dst + r) == (int32_t)v) {
    c += cnt[r];
    cnt[r] = c;
  }
  cnt[e] = c;
}

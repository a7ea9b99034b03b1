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

// ids per lane in a full piece of a long probe list (two per 8-byte load); at R-MAT
// scale 24, 8 measured 4% slower
#define LONG_UNROLL 16

// pre[u] = |N(u) ∩ [0, u)|; vinfo (optional) = (off[u], pre[u]) packed, so that a
// kernel looking up a random partner reads one 8-byte record instead of two arrays
// (on graphs without locality, e.g. Erdos-Renyi, each lookup is a DRAM access).
__global__ void k_pre(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst, uint32_t n,
                      uint32_t *__restrict__ pre, uint2 *__restrict__ vinfo) {
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const uint32_t b = __ldg(off + u), e = __ldg(off + u + 1);
    const uint32_t p = accx_lower_bound(dst, b, e, (int32_t)u) - b;
    pre[u] = p;
    if (vinfo) vinfo[u] = make_uint2(b, p);
  }
}

// Reverse entries: rev[e] = position of u in N(v) for every entry e = (u,v).
// One thread per entry e = (v,u) with u > v searches v in u's prefix (a short
// list after the degree relabel) and sets both directions; entries without a
// reverse (asymmetric input) keep the 0xffffffff the array was filled with.
template <int TILE>
__global__ void __launch_bounds__(TILE) k_rev_build(const uint32_t *__restrict__ off,
                                                    const uint32_t *__restrict__ tilerow,
                                                    const int32_t *__restrict__ dst,
                                                    const uint32_t *__restrict__ pre, uint32_t n, uint32_t m,
                                                    uint32_t *__restrict__ rev) {
  __shared__ accx_tile_rows<TILE> sh;
  const uint32_t base = blockIdx.x * (uint32_t)TILE;
  const uint32_t e = base + threadIdx.x;
  const uint32_t v = accx_tile_row<TILE>(off, tilerow, n, m, base, e, &sh);
  if (e >= m) return;
  const uint32_t u = (uint32_t)dst[e];
  if (u <= v) return;
  const uint32_t ub = __ldg(off + u), ue = ub + __ldg(pre + u);
  const uint32_t r = accx_lower_bound(dst, ub, ue, (int32_t)v);
  if (r < ue && __ldg(dst + r) == (int32_t)v) {
    rev[e] = r;
    rev[r] = e;
  }
}

// The two prefix ranges of an owned edge (x owner, y = dst[e]), each cut at
// min(x, y): ids from there up cannot be common to both prefixes.  The cut of
// P(x) at y < x is the entry e itself; the cut of P(y) at x < y is x's position
// in N(y), the reverse entry.
__device__ __forceinline__ void accx_or_ranges(const uint32_t *__restrict__ off, const uint32_t *__restrict__ pre,
                                               const uint32_t *__restrict__ rev, uint32_t x, uint32_t y, uint32_t e,
                                               uint32_t *xb, uint32_t *xe, uint32_t *yb, uint32_t *ye) {
  *xb = __ldg(off + x);
  *xe = *xb + __ldg(pre + x);
  *yb = __ldg(off + y);
  *ye = *yb + __ldg(pre + y);
  if (y < x) {
    *xe = min(*xe, e);
  } else {
    const uint32_t r = __ldg(rev + e);
    *ye = (r >= *yb && r < *ye) ? r : *yb;
  }
}

__global__ void __launch_bounds__(MERGE_WARPS * 32) k_merge_or(const uint32_t *__restrict__ off,
                                                                const int32_t *__restrict__ dst,
                                                                const uint32_t *__restrict__ pre,
                                                                const uint32_t *__restrict__ rev,
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
    accx_or_ranges(off, pre, rev, x, y, e, &xb, &xe, &yb, &ye);
    const uint32_t c = accx_warp_merge_credit(dst, xb, xe, yb, ye, buf[w][0], buf[w][1], lane, cnt);
    if (lane == 0 && c) atomicAdd(cnt + (y < x ? e : ye), (int32_t)c);  // the edge's prefix entry
    found += c;
    __syncwarp();
  }
  if (lane == 0 && found) atomicAdd(&ctr[C_MATCH + ACCX_KIND_MERGE], found);
}

// Groups of G lanes take one edge each: the lanes take the partner's prefix ids
// in order and binary-search each in the owner's prefix; every round starts at
// the position the group's last lane reached.  Galloping edges mostly have
// short partner lists (the low-degree owners outside the bitmap window), so a
// warp works on 32/G edges at once.  The partner range comes from classify
// (sl[e], already cut at min(x, y)), so an edge needs its list record, that
// range and the owner's offset and prefix length (vinfo): y < x exactly when e lies in
// x's prefix, and then the owner's range is cut at e and the edge's credit goes
// to e; otherwise to the end of the partner range (x's position in N(y)).
template <int G>
__global__ void __launch_bounds__(MERGE_WARPS * 32) k_gallop_or(const uint2 *__restrict__ vinfo,
                                                                 const int32_t *__restrict__ dst,
                                                                 const uint2 *__restrict__ sl,
                                                                 const uint2 *__restrict__ list, uint32_t list_cap,
                                                                 unsigned long long *__restrict__ ctr,
                                                                 int32_t *__restrict__ cnt) {
  static_assert(G == 8 || G == 16 || G == 32, "group size");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int sub = lane / G, gl = lane % G;
  const unsigned gmask = G == 32 ? ACCX_FULL_MASK : (((1u << G) - 1u) << (sub * G));
  unsigned long long found = 0;
  unsigned long long total = ctr[C_GALLOP];
  if (total > list_cap) total = list_cap;
  const unsigned long long ng = (unsigned long long)gridDim.x * MERGE_WARPS * (32 / G);
  for (unsigned long long it = ((unsigned long long)blockIdx.x * MERGE_WARPS + w) * (32 / G) + sub; it < total;
       it += ng) {
    const uint2 p = list[list_cap - 1 - it];
    const uint32_t x = p.x, e = p.y;
    const uint2 r = __ldg(sl + e), xi = __ldg(vinfo + x);
    const uint32_t xb = xi.x, xp = xi.x + xi.y;
    const uint32_t xe = min(xp, e), yb = r.x, ye = r.x + (r.y & ~OR_SL_GALLOP);
    uint32_t c = 0, lo = xb;
    for (uint32_t j0 = yb; j0 < ye && lo < xe; j0 += G) {
      const uint32_t j = j0 + (uint32_t)gl;
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
      const uint32_t last = (ye - j0 >= (uint32_t)G) ? (uint32_t)G - 1u : (ye - j0 - 1);
      lo = __shfl_sync(gmask, pos, (int)last, G);
    }
#pragma unroll
    for (int d = G / 2; d >= 1; d >>= 1) c += __shfl_xor_sync(gmask, c, d, G);
    if (gl == 0 && c) atomicAdd(cnt + (e < xp ? e : ye), (int32_t)c);  // the edge's prefix entry
    if (gl == 0) found += c;
  }
  if (gl == 0 && found) atomicAdd(&ctr[C_MATCH + ACCX_KIND_GALLOP], found);
}

// items[i] = the owner of bitmap work item i (items of one owner are contiguous).
__global__ void k_item_fill(const unsigned long long *__restrict__ icnt, const unsigned long long *__restrict__ prefix,
                            uint32_t n, uint32_t cap, uint32_t *__restrict__ items) {
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const unsigned long long c = icnt[u], p0 = prefix[u];
    for (unsigned long long j = 0; j < c && p0 + j < cap; j++) items[p0 + j] = u;
  }
}

// One piece of a long list for one warp: G pair groups (64 G ids) from the
// even entry j0.  Lane pairs (j, j+1) come from one 8-byte load; ids outside
// [a0, a1) are dropped (the array's padding keeps the last pair in bounds).
// Every load is issued before the probes (a test per load would serialise
// them); the probes stop at the first pair group past the list end.  A hit at
// entry j credits cnt[j] -- a warp's credits for one load land in one line of
// cnt -- and the owner counter of the id's rank; returns this lane's hits.
template <int G>
__device__ __forceinline__ uint32_t or_piece(const int32_t *__restrict__ dst, uint32_t j0, uint32_t a0, uint32_t a1,
                                             uint32_t lane, uint32_t W, const uint32_t *words, const uint16_t *wbase,
                                             uint32_t *ocnt, uint32_t pxs, int32_t *__restrict__ cnt) {
  const uint32_t rem = a1 - j0;
  int2 v[G];
#pragma unroll
  for (int r = 0; r < G; r++) {
    const uint32_t j = j0 + 64u * r + 2u * lane;
    v[r] = j < a1 ? __ldg(reinterpret_cast<const int2 *>(dst + j)) : make_int2(-1, -1);
    if (j < a0) v[r].x = -1;
    if (j + 1u >= a1) v[r].y = -1;
  }
  int32_t *const cl = cnt + j0 + 2u * lane;
  uint32_t h = 0;
#pragma unroll
  for (int r = 0; r < 2 * G; r++) {
    if (64u * (uint32_t)(r >> 1) >= rem) break;
    const uint32_t id = min((uint32_t)((r & 1) ? v[r >> 1].y : v[r >> 1].x), W);  // W: the zero word
    const uint32_t wd = words[id >> 5];
    if ((wd >> (id & 31u)) & 1u) {
      // the rank: the word's base plus the set bits up to and including this one, less one
      const uint32_t rk = wbase[id >> 5] + __popc(wd << (~id & 31u)) - 1u;
      h++;
      atomicAdd(cl + 64u * (r >> 1) + (uint32_t)(r & 1), 1);
      atomicAdd(&ocnt[rk], 1u);  // rk < pxs on a sorted CSR, < pxs + 31 always (spare counters)
    }
  }
  return h;
}

#define SHORT_PIECE (32u * PROBE_UNROLL)  // ids per short piece (concatenated short lists)
#define LONG_PIECE (32u * LONG_UNROLL)    // ids per piece of a long list

// Bitmap kind.  CTAs take work items (an owner x, or a slice of its list when
// the owner's probe work is large) from a device counter.  The owner's prefix
// -- ids below x, which the classifier keeps below W -- is staged as a dense
// bitmap over [0, W) plus, per non-empty 32-bit word, the prefix position of
// the word's first id (rank of an id = that base + popcount of the lower bits).
// The slice is walked in rounds of blockDim entries; the classifier stored, per
// bitmap entry (x,y), where P(y) starts and its length cut at min(x,y) (0 for
// other entries), so a round starts with one coalesced load per entry.  Short
// probe lists are concatenated (CTA prefix sum) and cut into chunks; warps take
// whole long lists (at most the owner counters' size, walked in pieces of
// LONG_PIECE ids) and then the short chunks from one shared queue, so the
// small grains even out the round's end.  A hit at partner entry j
// credits cnt[j] (RED), the owner's shared counter of the id's rank, and the
// edge (shared per-entry counters, credited after the round).
// NT = the block size the per-round arrays are sized for (blockDim.x <= NT); a
// 512-thread instance needs half the static shared memory, so two CTAs fit an
// SM when the window is small enough, and a 256-thread one with a small window
// runs four per SM.
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_bitmap_or(const uint32_t *__restrict__ off,
                                                       const int32_t *__restrict__ dst,
                                                       const uint32_t *__restrict__ pre, uint32_t n,
                                                       const uint32_t *__restrict__ items, uint32_t items_cap,
                                                       const unsigned long long *__restrict__ work_u,
                                                       const unsigned long long *__restrict__ prefix,
                                                       const uint2 *__restrict__ sl, uint32_t W, uint32_t pcap,
                                                       uint32_t target, int32_t *__restrict__ cnt,
                                                       unsigned long long *__restrict__ ctr) {
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t nwords = W / 32;
  uint32_t *words = smem;                                          // nwords + a zero word (ids >= W probe it)
  // pcap owner-prefix counters + 32 spares: a found id's rank is at most a word's
  // base (< pxs) + 31, so the counter add needs no bounds test even on unsorted input
  uint32_t *ocnt = smem + nwords + 4;
  uint16_t *wbase = reinterpret_cast<uint16_t *>(ocnt + pcap + 32);  // nwords first-id positions
  __shared__ unsigned long long s_it;
  __shared__ uint32_t s_tot, s_nseg, s_nlong, s_next;
  __shared__ uint32_t s_wsum[32], s_wcnt[32], s_wlong[32];
  __shared__ uint32_t s_pre[NT + 1], s_beg[NT], s_ent[NT], s_hit[NT];
  __shared__ uint32_t s_lbeg[NT], s_llen[NT], s_lent[NT], s_lhit[NT];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  for (uint32_t i = tid; i <= nwords; i += nt) words[i] = 0;
  unsigned long long total = prefix[n];
  if (total > items_cap) total = items_cap;
  unsigned long long found = 0, probed = 0;  // this thread's share, summed per warp at the end
  if (tid == 0) s_it = atomicAdd(&ctr[C_ITEMS], 1ull);
  __syncthreads();
  for (;;) {
    const unsigned long long it = s_it;
    if (it >= total) break;
    const uint32_t x = items[it];
    const uint32_t ub = off[x], ue = off[x + 1], du = ue - ub, px = pre[x];
    uint32_t nchunks, nsplit;
    accx_item_shape(du, 0, work_u[x], 1, target, &nchunks, &nsplit);
    const uint32_t sp = (uint32_t)(it - prefix[x]);
    const uint32_t pa = ub + (uint32_t)((unsigned long long)du * sp / nsplit);
    const uint32_t pb = ub + (uint32_t)((unsigned long long)du * (sp + 1) / nsplit);
    const uint32_t pxs = px <= pcap ? px : 0;  // the classifier guarantees px <= pcap for bitmap owners
    for (uint32_t i = tid; i < pxs; i += nt) {
      const uint32_t id = (uint32_t)__ldg(dst + ub + i);
      if (id < W) {
        atomicOr(&words[id >> 5], 1u << (id & 31));
        if (i == 0 || ((uint32_t)__ldg(dst + ub + i - 1) >> 5) != (id >> 5)) wbase[id >> 5] = (uint16_t)i;
      }
      ocnt[i] = 0;
    }
    __syncthreads();
    if (tid == 0) s_it = atomicAdd(&ctr[C_ITEMS], 1ull);  // the next item, read after this one
    for (uint32_t r0 = pa; r0 < pb; r0 += (uint32_t)nt) {
      const uint32_t k = r0 + (uint32_t)tid;
      uint32_t sst = 0, len = 0;
      if (k < pb) {
        const uint2 e = sl[k];
        sst = e.x;
        len = (e.y & OR_SL_GALLOP) ? 0u : e.y;  // galloping entries are not this kernel's
      }
      probed += len;
      const bool is_short = len > 0 && len < LONG_SEG, is_long = len >= LONG_SEG;
      const unsigned bs = __ballot_sync(ACCX_FULL_MASK, is_short), bl = __ballot_sync(ACCX_FULL_MASK, is_long);
      uint32_t incl = is_short ? len : 0u;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t a = __shfl_up_sync(ACCX_FULL_MASK, incl, d);
        if (lane >= d) incl += a;
      }
      if (lane == 31) {
        s_wsum[warp] = incl;
        s_wcnt[warp] = __popc(bs);
        s_wlong[warp] = __popc(bl);
      }
      __syncthreads();
      if (warp == 0) {
        const uint32_t ws = lane < nwarps ? s_wsum[lane] : 0u, wc = lane < nwarps ? s_wcnt[lane] : 0u;
        const uint32_t wl = lane < nwarps ? s_wlong[lane] : 0u;
        uint32_t is = ws, ic = wc, il = wl;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const uint32_t a = __shfl_up_sync(ACCX_FULL_MASK, is, d), b = __shfl_up_sync(ACCX_FULL_MASK, ic, d);
          const uint32_t c = __shfl_up_sync(ACCX_FULL_MASK, il, d);
          if (lane >= d) { is += a; ic += b; il += c; }
        }
        if (lane < nwarps) {
          s_wsum[lane] = is - ws;
          s_wcnt[lane] = ic - wc;
          s_wlong[lane] = il - wl;
        }
        if (lane == 31) { s_tot = is; s_nseg = ic; s_nlong = il; s_next = 0; }
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
        s_lhit[idx] = 0;
      }
      if (tid == 0) s_pre[s_nseg] = s_tot;
      __syncthreads();
      const uint32_t tot = s_tot, nseg = s_nseg, nlong = s_nlong;
      // the queue: whole long lists first (the larger grains), then short chunks
      const uint32_t nsp = (tot + SHORT_PIECE - 1) / SHORT_PIECE, npieces = nlong + nsp;
      for (;;) {
        uint32_t p = 0;
        if (lane == 0) p = atomicAdd(&s_next, 1u);
        p = __shfl_sync(ACCX_FULL_MASK, p, 0);
        if (p >= npieces) break;
        if (p >= nlong) {
          // short chunk: SHORT_PIECE consecutive ids of the concatenation
          const uint32_t c0 = (p - nlong) * SHORT_PIECE;
          uint32_t lo = 0, hi = nseg;
          while (hi - lo > 1) {
            const uint32_t step = (hi - lo + 31) / 32;
            const uint32_t q = lo + (uint32_t)lane * step;
            const unsigned b = __ballot_sync(ACCX_FULL_MASK, q < hi && s_pre[q] <= c0);
            lo += (31 - __clz(b)) * step;
            const uint32_t nh = lo + step;
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
            // ids >= W (the -1 of lanes past the end) read the zero word
            const uint32_t id = min((uint32_t)xs[r], W);
            const uint32_t wd = words[id >> 5];
            if ((wd >> (id & 31u)) & 1u) {
              const uint32_t rk = wbase[id >> 5] + __popc(wd << (~id & 31u)) - 1u;
              atomicAdd(cnt + gi[r], 1);
              atomicAdd(&ocnt[rk], 1u);  // rk < pxs on a sorted CSR, < pxs + 31 always (spare counters)
              atomicAdd(&s_hit[sg[r]], 1u);
            }
          }
        } else {
          // a long list, walked in pieces of LONG_PIECE ids from the even entry at
          // or before its start
          const uint32_t q = p;
          const uint32_t a0 = s_lbeg[q], a1 = a0 + s_llen[q];
          uint32_t h = 0;
          for (uint32_t j0 = a0 & ~1u; j0 < a1; j0 += LONG_PIECE) {
            // the last piece loads only the pair groups it needs (the size
            // class is warp-uniform, and each class issues all its loads at once)
            const uint32_t rem = a1 - j0;
            if (rem > 256u) h += or_piece<LONG_UNROLL / 2>(dst, j0, a0, a1, lane, W, words, wbase, ocnt, pxs, cnt);
            else if (rem > 128u) h += or_piece<4>(dst, j0, a0, a1, lane, W, words, wbase, ocnt, pxs, cnt);
            else if (rem > 64u) h += or_piece<2>(dst, j0, a0, a1, lane, W, words, wbase, ocnt, pxs, cnt);
            else h += or_piece<1>(dst, j0, a0, a1, lane, W, words, wbase, ocnt, pxs, cnt);
          }
          h = __reduce_add_sync(ACCX_FULL_MASK, h);
          if (lane == 0 && h) atomicAdd(&s_lhit[q], h);
        }
      }
      __syncthreads();
      // edge credits go to the edge's prefix entry: the entry itself when y < x
      // (through the owner's counters), else x's position in N(y), which is where
      // the partner range was cut
      for (uint32_t q = tid; q < nseg + nlong; q += nt) {
        const bool sh = q < nseg;
        const uint32_t h = sh ? s_hit[q] : s_lhit[q - nseg], kk = sh ? s_ent[q] : s_lent[q - nseg];
        found += h;
        if (h) {
          if (kk - ub < px) {
            if (kk - ub < pxs) atomicAdd(&ocnt[kk - ub], h);
            else atomicAdd(cnt + kk, (int32_t)h);
          } else {
            const uint32_t cut = sh ? s_beg[q] + (s_pre[q + 1] - s_pre[q]) : s_lbeg[q - nseg] + s_llen[q - nseg];
            atomicAdd(cnt + cut, (int32_t)h);
          }
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

// Every credit lands on an edge's prefix entry (the entry in the larger id's
// list), which starts at the bias (written by classify); the other entry copies
// it.  One thread per entry: a suffix entry e = (v,u), u > v, takes the count of its
// reverse rev[e] > e (u's prefix entry); entries without a reverse (asymmetric
// input) keep the bias.
__global__ void k_combine_or(uint32_t m, const uint32_t *__restrict__ rev, int32_t *__restrict__ cnt) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  const uint32_t r = rev[e];
  if (r != 0xffffffffu && r > e) cnt[e] = cnt[r];
}


// Degree-descending relabel of a resident graph, on the GPU.
//
// The reference offers the same preprocessing on the CPU (ReorderDegDescending +
// Reorder, scan-query/scan_xp.cpp:1145-1222, :1279-1301): vertices are renumbered
// by decreasing degree and every neighbour list is re-sorted.  Here it serves the
// counting kernels: after the relabel most probed ids (edge endpoints are mostly
// high-degree vertices) are small, so a dense shared-memory bitmap over the
// lowest ids answers most membership tests.  Counts are computed on the relabeled
// CSR and gathered back to the caller's entry order through map[e], so the
// handle's public arrays never change.
#include <cub/cub.cuh>

#include "accx_internal.h"
#include "devutil.cuh"

__global__ void k_vertex_keys(const uint32_t *__restrict__ off, uint32_t n, unsigned long long *__restrict__ keys) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    uint32_t d = off[v + 1] - off[v];
    keys[v] = ((unsigned long long)(0xffffffffu - d) << 32) | v;  // degree descending, then id
  }
}

__global__ void k_perm(const unsigned long long *__restrict__ sorted, uint32_t n, const uint32_t *__restrict__ off,
                       uint32_t *__restrict__ oldid, uint32_t *__restrict__ newid, uint32_t *__restrict__ rdeg) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t v = (uint32_t)(sorted[i] & 0xffffffffull);
    oldid[i] = v;
    newid[v] = i;
    rdeg[i] = off[v + 1] - off[v];
  }
}

// Rows move whole: the row of old vertex u becomes row newid[u], so an entry's
// new place is that row's start plus its old position in the row; it carries the
// new id of its neighbour (the sort key) and its own old index.  Rows are sorted
// by key afterwards.
template <int TILE>
__global__ void __launch_bounds__(TILE) k_row_scatter(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow,
                                                      const int32_t *__restrict__ dst, uint32_t n, uint32_t m,
                                                      const uint32_t *__restrict__ newid, const uint32_t *__restrict__ roff,
                                                      uint32_t *__restrict__ key, uint32_t *__restrict__ val) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, tilerow, n, m, base, e, &sh);
  if (e >= m) return;
  const uint32_t p = roff[newid[u]] + (e - off[u]);
  const uint32_t v = (uint32_t)dst[e];
  key[p] = v < n ? newid[v] : 0xffffffffu;
  val[p] = e;
}

// Relabeled rows are in non-increasing degree order, so each degree class is a
// range of rows: bounds[i] = the first row of degree <= RELABEL_CLASS[i].
#define RELABEL_NCLASS 5
__constant__ uint32_t RELABEL_CLASS[RELABEL_NCLASS] = {4096u, 1024u, 256u, 32u, 1u};

__global__ void k_class_bounds(const uint32_t *__restrict__ rdeg, uint32_t n, uint32_t *__restrict__ bounds) {
  const int i = threadIdx.x;
  if (i >= RELABEL_NCLASS) return;
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (rdeg[mid] <= RELABEL_CLASS[i]) hi = mid;
    else lo = mid + 1;
  }
  bounds[i] = lo;
}

// Writes sorted row entries: the relabeled neighbour id and, for the entry's old
// index, its new position.
__device__ __forceinline__ void relabel_put(uint32_t p, uint32_t k, uint32_t v, int32_t *__restrict__ rdst,
                                            uint32_t *__restrict__ map) {
  rdst[p] = (int32_t)k;
  map[v] = p;
}

// One CTA per row of at most NT*IPT entries (rows r0..r1, CTAs loop over them):
// block radix sort over the low `bits` bits.  Padding keys are all ones and
// `bits` leaves them above every id, so they sort last.  The input arrangement
// does not matter to the sort, so loads are striped (coalesced).
template <int NT, int IPT>
__global__ void __launch_bounds__(NT) k_row_sort(uint32_t r0, uint32_t r1, const uint32_t *__restrict__ roff,
                                                 const uint32_t *__restrict__ key, const uint32_t *__restrict__ val,
                                                 int bits, int32_t *__restrict__ rdst, uint32_t *__restrict__ map) {
  using Sort = cub::BlockRadixSort<uint32_t, NT, IPT, uint32_t, 5>;  // 5-bit digits: 4 and 6 measured slower
  __shared__ typename Sort::TempStorage tmp;
  for (uint32_t r = r0 + blockIdx.x; r < r1; r += gridDim.x) {
    const uint32_t b = roff[r], d = roff[r + 1] - b;
    uint32_t k[IPT], v[IPT];
#pragma unroll
    for (int i = 0; i < IPT; i++) {
      const uint32_t idx = (uint32_t)i * NT + threadIdx.x;
      k[i] = idx < d ? key[b + idx] : 0xffffffffu;
      v[i] = idx < d ? val[b + idx] : 0u;
    }
    Sort(tmp).SortBlockedToStriped(k, v, 0, bits);
#pragma unroll
    for (int i = 0; i < IPT; i++) {
      const uint32_t idx = (uint32_t)i * NT + threadIdx.x;
      if (idx < d) relabel_put(b + idx, k[i], v[i], rdst, map);
    }
    __syncthreads();  // tmp is reused by the next row
  }
}

// One warp per row of at most 32 entries: bitonic sort across the lanes.
__global__ void k_warp_row_sort(uint32_t r0, uint32_t r1, const uint32_t *__restrict__ roff,
                                const uint32_t *__restrict__ key, const uint32_t *__restrict__ val,
                                int32_t *__restrict__ rdst, uint32_t *__restrict__ map) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = r0 + w; r < r1; r += nw) {
    const uint32_t b = roff[r], d = roff[r + 1] - b;
    uint32_t k = lane < d ? key[b + lane] : 0xffffffffu, v = lane < d ? val[b + lane] : 0u;
#pragma unroll
    for (uint32_t sz = 2; sz <= 32; sz <<= 1) {
#pragma unroll
      for (uint32_t j = sz >> 1; j > 0; j >>= 1) {
        const uint32_t ok = __shfl_xor_sync(ACCX_FULL_MASK, k, j), ov = __shfl_xor_sync(ACCX_FULL_MASK, v, j);
        // ascending runs of sz lanes alternate with descending ones; the lower
        // lane of a pair keeps the smaller key in an ascending run
        const bool keep_min = ((lane & j) == 0) == ((lane & sz) == 0);
        if (keep_min ? (ok < k) : (ok > k)) {
          k = ok;
          v = ov;
        }
      }
    }
    if (lane < d) relabel_put(b + lane, k, v, rdst, map);
  }
}

// Entries [p0, p1) that are already in order (rows of at most one entry, or rows
// sorted by the segmented sort).
__global__ void k_put_range(const uint32_t *__restrict__ key, const uint32_t *__restrict__ val, uint32_t p0,
                            uint32_t p1, int32_t *__restrict__ rdst, uint32_t *__restrict__ map) {
  for (uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x; p < p1; p += gridDim.x * blockDim.x)
    relabel_put(p, key[p], val[p], rdst, map);
}

// Four entries per thread and step, their index loads and then their gathers
// issued together: the gathers are random reads, bound by latency at one a thread.
// host (optional): the caller's pinned output buffer mapped into the device's
// address space, written in the same pass (each warp store is 128 contiguous
// bytes over the host link), which spares a separate copy of the counts.
__global__ void k_gather_counts(const int32_t *__restrict__ cnt_r, const uint32_t *__restrict__ map, uint32_t m,
                                int32_t *__restrict__ cnt, int32_t *__restrict__ host) {
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  for (; e + 3 * stride < m; e += 4 * stride) {
    const uint32_t a = __ldg(map + e), b = __ldg(map + e + stride), c = __ldg(map + e + 2 * stride),
                   d = __ldg(map + e + 3 * stride);
    const int32_t x = __ldg(cnt_r + a), y = __ldg(cnt_r + b), z = __ldg(cnt_r + c), w = __ldg(cnt_r + d);
    cnt[e] = x;
    cnt[e + stride] = y;
    cnt[e + 2 * stride] = z;
    cnt[e + 3 * stride] = w;
    if (host) {
      host[e] = x;
      host[e + stride] = y;
      host[e + 2 * stride] = z;
      host[e + 3 * stride] = w;
    }
  }
  for (; e < m; e += stride) {
    const int32_t x = __ldg(cnt_r + __ldg(map + e));
    cnt[e] = x;
    if (host) host[e] = x;
  }
}

int accx_relabel_gather(accx_graph *g, int32_t *host, cudaStream_t s) {
  const uint32_t m = (uint32_t)g->m;
  if (!m) return ACCX_OK;
  k_gather_counts<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(g->d_rcnt, g->d_rmap, m, g->d_cnt, host);
  ACCX_CUDA_TRY(cudaGetLastError());
  return ACCX_OK;
}

extern "C" int accx_graph_relabel(accx_graph *g, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  if (g->d_roff) return ACCX_OK;
  cudaStream_t s = (cudaStream_t)stream;
  ACCX_CUDA_TRY(cudaSetDevice(g->device));
  const uint32_t n = g->n, m = (uint32_t)g->m;
  const int grid = accx_sm_count(g->device) * 8;
  unsigned long long *vkeys = nullptr, *vkeys2 = nullptr;
  uint32_t *key = nullptr, *val = nullptr, *key2 = nullptr, *val2 = nullptr, *rdeg = nullptr, *bounds = nullptr;
  void *tmp = nullptr;
  size_t tb = 0;
  int rc = ACCX_OK;
  do {
    if (accx_dev_alloc((void **)&vkeys, sizeof(unsigned long long) * ((size_t)n + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&vkeys2, sizeof(unsigned long long) * ((size_t)n + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&key, sizeof(uint32_t) * ((size_t)m + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&val, sizeof(uint32_t) * ((size_t)m + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&rdeg, sizeof(uint32_t) * ((size_t)n + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&bounds, sizeof(uint32_t) * 8, g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&g->d_roff, sizeof(uint32_t) * ((size_t)n + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&g->d_rdst, sizeof(int32_t) * ((size_t)m + ACCX_DST_PAD), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&g->d_rmap, sizeof(uint32_t) * ((size_t)m + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&g->d_rcnt, sizeof(int32_t) * ((size_t)m + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&g->d_oldid, sizeof(uint32_t) * ((size_t)n + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&g->d_newid, sizeof(uint32_t) * ((size_t)n + 1), g->home) != cudaSuccess) {
      rc = ACCX_ERR_OOM;
      break;
    }
    if (g->home && cudaStreamSynchronize(g->home) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    // sort keys: ids need `bits` bits with the all-ones pattern left above every id
    int bits = 1;
    while (bits < 32 && (1ull << bits) <= (unsigned long long)n) bits++;
    cub::DoubleBuffer<unsigned long long> dk(vkeys, vkeys2);
    size_t b1 = 0, b2 = 0;
    if (cub::DeviceRadixSort::SortKeys(nullptr, b1, dk, (int64_t)n, 0, 64, s) != cudaSuccess ||
        cub::DeviceScan::ExclusiveSum(nullptr, b2, rdeg, g->d_roff, (int64_t)n + 1, s) != cudaSuccess) {
      rc = ACCX_ERR_CUDA;
      break;
    }
    tb = b1 > b2 ? b1 : b2;
    if (accx_dev_alloc(&tmp, tb + 16, g->home) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    if (g->home && cudaStreamSynchronize(g->home) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    // 1. vertex order: degree descending, ties by id
    if (n) {
      k_vertex_keys<<<grid, 256, 0, s>>>(g->d_off, n, vkeys);
      if (cub::DeviceRadixSort::SortKeys(tmp, tb, dk, (int64_t)n, 0, 64, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
      k_perm<<<grid, 256, 0, s>>>(dk.Current(), n, g->d_off, g->d_oldid, g->d_newid, rdeg);
    }
    if (cudaMemsetAsync(rdeg + n, 0, sizeof(uint32_t), s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (cub::DeviceScan::ExclusiveSum(tmp, tb, rdeg, g->d_roff, (int64_t)n + 1, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (m) {
      // 2. rows to their new places, keyed by the neighbours' new ids
      k_row_scatter<256><<<(m + 255) / 256, 256, 0, s>>>(g->d_off, g->d_tilerow, g->d_dst, n, m, g->d_newid,
                                                         g->d_roff, key, val);
      // 3. sort every row by key, with a kernel sized for its degree class
      uint32_t hb[2 * RELABEL_NCLASS];
      k_class_bounds<<<1, 32, 0, s>>>(rdeg, n, bounds);
      if (cudaMemcpyAsync(hb, bounds, sizeof(uint32_t) * RELABEL_NCLASS, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) {
        rc = ACCX_ERR_CUDA;
        break;
      }
      for (int i = 0; i < RELABEL_NCLASS; i++)
        if (cudaMemcpyAsync(hb + RELABEL_NCLASS + i, g->d_roff + hb[i], sizeof(uint32_t), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess) rc = ACCX_ERR_CUDA;
      if (rc || cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
      const uint32_t *rb = hb, *pb = hb + RELABEL_NCLASS;  // class row bounds and their entry positions
      const int sms = accx_sm_count(g->device);
      // rows above 4096 entries: segmented radix sort (one CTA per row)
      if (rb[0] > 0) {
        size_t b3 = 0;
        if (cub::DeviceSegmentedRadixSort::SortPairs(nullptr, b3, key, key, val, val, (int64_t)pb[0], (int64_t)rb[0],
                                                     g->d_roff, g->d_roff + 1, 0, bits, s) != cudaSuccess) {
          rc = ACCX_ERR_CUDA;
          break;
        }
        if (b3 > tb) {
          if (cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
          accx_dev_free(tmp, g->home);
          tmp = nullptr;
          tb = b3;
          if (accx_dev_alloc(&tmp, tb + 16, g->home) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
          if (g->home && cudaStreamSynchronize(g->home) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
        }
        if (accx_dev_alloc((void **)&key2, sizeof(uint32_t) * ((size_t)pb[0] + 1), g->home) != cudaSuccess ||
            accx_dev_alloc((void **)&val2, sizeof(uint32_t) * ((size_t)pb[0] + 1), g->home) != cudaSuccess) {
          rc = ACCX_ERR_OOM;
          break;
        }
        if (g->home && cudaStreamSynchronize(g->home) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
        if (cub::DeviceSegmentedRadixSort::SortPairs(tmp, tb, key, key2, val, val2, (int64_t)pb[0], (int64_t)rb[0],
                                                     g->d_roff, g->d_roff + 1, 0, bits, s) != cudaSuccess) {
          rc = ACCX_ERR_CUDA;
          break;
        }
        k_put_range<<<sms * 8, 256, 0, s>>>(key2, val2, 0u, pb[0], g->d_rdst, g->d_rmap);
      }
      auto rows_grid = [&](uint32_t rows, int per_sm) { return (int)(rows < (uint32_t)(sms * per_sm) ? rows : sms * per_sm); };
      if (rb[1] > rb[0])
        k_row_sort<256, 16><<<rows_grid(rb[1] - rb[0], 8), 256, 0, s>>>(rb[0], rb[1], g->d_roff, key, val, bits,
                                                                           g->d_rdst, g->d_rmap);
      if (rb[2] > rb[1])
        k_row_sort<128, 8><<<rows_grid(rb[2] - rb[1], 16), 128, 0, s>>>(rb[1], rb[2], g->d_roff, key, val, bits,
                                                                          g->d_rdst, g->d_rmap);
      if (rb[3] > rb[2])
        k_row_sort<64, 4><<<rows_grid(rb[3] - rb[2], 32), 64, 0, s>>>(rb[2], rb[3], g->d_roff, key, val, bits,
                                                                        g->d_rdst, g->d_rmap);
      if (rb[4] > rb[3])
        k_warp_row_sort<<<rows_grid((rb[4] - rb[3] + 7) / 8, 16), 256, 0, s>>>(rb[3], rb[4], g->d_roff, key, val,
                                                                                g->d_rdst, g->d_rmap);
      if (m > pb[4]) k_put_range<<<sms * 8, 256, 0, s>>>(key, val, pb[4], m, g->d_rdst, g->d_rmap);
    }
    if (cudaMemsetAsync(g->d_rdst + m, 0xff, sizeof(int32_t) * ACCX_DST_PAD, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if ((rc = accx_tilerow_build(g, g->d_roff, &g->d_rtilerow, s)) != ACCX_OK) break;
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
  } while (0);
  if (rc) {
    cudaGetLastError();
    cudaStreamSynchronize(s);  // nothing of this call may still be running on the temporaries
  }
  for (void *p : {(void *)vkeys, (void *)vkeys2, (void *)key, (void *)val, (void *)key2, (void *)val2, (void *)rdeg,
                  (void *)bounds, tmp})
    accx_dev_free(p, g->home);
  if (!rc && g->d_rev_orig) {  // counts run on the relabeled CSR from now on
    accx_dev_free(g->d_rev_orig, g->home);
    g->d_rev_orig = nullptr;
  }
  if (rc) {
    for (void **p : {(void **)&g->d_roff, (void **)&g->d_rdst, (void **)&g->d_rmap, (void **)&g->d_rcnt,
                     (void **)&g->d_oldid, (void **)&g->d_newid, (void **)&g->d_rtilerow}) {
      accx_dev_free(*p, g->home);
      *p = nullptr;
    }
  }
  return rc;
}

extern "C" int accx_graph_is_relabeled(const accx_graph *g) { return g && g->d_roff ? 1 : 0; }

extern "C" int accx_graph_relabeled_csr(const accx_graph *g, uint32_t *roff, int32_t *rdst, uint32_t *map,
                                        uint32_t *oldid, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  if (!g->d_roff) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = ACCX_OK;
  if (!rc && roff) rc = accx_copy_out(roff, g->d_roff, sizeof(uint32_t) * ((size_t)g->n + 1), s);
  if (!rc && rdst) rc = accx_copy_out(rdst, g->d_rdst, sizeof(int32_t) * (size_t)g->m, s);
  if (!rc && map) rc = accx_copy_out(map, g->d_rmap, sizeof(uint32_t) * (size_t)g->m, s);
  if (!rc && oldid) rc = accx_copy_out(oldid, g->d_oldid, sizeof(uint32_t) * (size_t)g->n, s);
  return rc;
}

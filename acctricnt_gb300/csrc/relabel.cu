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

template <int TILE>
__global__ void __launch_bounds__(TILE) k_entry_keys(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow, const int32_t *__restrict__ dst,
                                                     uint32_t n, uint32_t m, const uint32_t *__restrict__ newid,
                                                     int nb, unsigned long long *__restrict__ keys,
                                                     uint32_t *__restrict__ vals) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, tilerow, n, m, base, e, &sh);
  if (e >= m) return;
  keys[e] = ((unsigned long long)newid[u] << nb) | newid[(uint32_t)dst[e]];  // 2*nb significant bits
  vals[e] = e;
}

__global__ void k_unpack_entries(const unsigned long long *__restrict__ keys, const uint32_t *__restrict__ vals,
                                 uint32_t m, unsigned long long vmask, int32_t *__restrict__ rdst,
                                 uint32_t *__restrict__ map) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    rdst[i] = (int32_t)(keys[i] & vmask);
    map[vals[i]] = i;
  }
}

__global__ void k_gather_counts(const int32_t *__restrict__ cnt_r, const uint32_t *__restrict__ map, uint32_t m,
                                int32_t *__restrict__ cnt) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x)
    cnt[e] = __ldg(cnt_r + __ldg(map + e));
}

int accx_relabel_gather(accx_graph *g, cudaStream_t s) {
  const uint32_t m = (uint32_t)g->m;
  if (!m) return ACCX_OK;
  k_gather_counts<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(g->d_rcnt, g->d_rmap, m, g->d_cnt);
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
  unsigned long long *k1 = nullptr, *k2 = nullptr;
  uint32_t *v1 = nullptr, *v2 = nullptr, *rdeg = nullptr;
  void *tmp = nullptr;
  int rc = ACCX_OK;
  do {
    const size_t big = (size_t)(m > n ? m : n) + 1;
    if (accx_dev_alloc((void **)&k1, sizeof(unsigned long long) * big, g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&k2, sizeof(unsigned long long) * big, g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&v1, sizeof(uint32_t) * big, g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&v2, sizeof(uint32_t) * big, g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&rdeg, sizeof(uint32_t) * ((size_t)n + 1), g->home) != cudaSuccess ||
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
    // entry keys (new u, new v) need 2*nb bits, nb = bits of the largest id
    int nb = 1;
    while (nb < 32 && (1ull << nb) < (unsigned long long)n) nb++;
    size_t b1 = 0, b2 = 0, b3 = 0;
    cub::DoubleBuffer<unsigned long long> dk(k1, k2);
    cub::DoubleBuffer<uint32_t> dv(v1, v2);
    if (cub::DeviceRadixSort::SortKeys(nullptr, b1, dk, (int64_t)n, 0, 64, s) != cudaSuccess ||
        cub::DeviceRadixSort::SortPairs(nullptr, b2, dk, dv, (int64_t)m, 0, 2 * nb, s) != cudaSuccess ||
        cub::DeviceScan::ExclusiveSum(nullptr, b3, rdeg, g->d_roff, (int64_t)n + 1, s) != cudaSuccess) {
      rc = ACCX_ERR_CUDA;
      break;
    }
    size_t tb = b1 > b2 ? b1 : b2;
    tb = tb > b3 ? tb : b3;
    if (accx_dev_alloc(&tmp, tb + 16, g->home) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    if (g->home && cudaStreamSynchronize(g->home) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    // 1. vertex order
    if (n) {
      k_vertex_keys<<<grid, 256, 0, s>>>(g->d_off, n, k1);
      if (cub::DeviceRadixSort::SortKeys(tmp, tb, dk, (int64_t)n, 0, 64, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
      k_perm<<<grid, 256, 0, s>>>(dk.Current(), n, g->d_off, g->d_oldid, g->d_newid, rdeg);
    }
    if (cudaMemsetAsync(rdeg + n, 0, sizeof(uint32_t), s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (cub::DeviceScan::ExclusiveSum(tmp, tb, rdeg, g->d_roff, (int64_t)n + 1, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    // 2. entries: (new u, new v) keys carrying the original entry index
    dk = cub::DoubleBuffer<unsigned long long>(k1, k2);
    if (m) {
      k_entry_keys<256><<<(m + 255) / 256, 256, 0, s>>>(g->d_off, g->d_tilerow, g->d_dst, n, m, g->d_newid, nb, k1, v1);
      if (cub::DeviceRadixSort::SortPairs(tmp, tb, dk, dv, (int64_t)m, 0, 2 * nb, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
      k_unpack_entries<<<grid, 256, 0, s>>>(dk.Current(), dv.Current(), m, (1ull << nb) - 1ull, g->d_rdst, g->d_rmap);
    }
    if (cudaMemsetAsync(g->d_rdst + m, 0xff, sizeof(int32_t) * ACCX_DST_PAD, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if ((rc = accx_tilerow_build(g, g->d_roff, &g->d_rtilerow, s)) != ACCX_OK) break;
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
  } while (0);
  if (rc) {
    cudaGetLastError();
    cudaStreamSynchronize(s);  // nothing of this call may still be running on the temporaries
  }
  for (void *p : {(void *)k1, (void *)k2, (void *)v1, (void *)v2, (void *)rdeg, tmp}) accx_dev_free(p, g->home);
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

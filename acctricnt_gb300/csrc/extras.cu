// Edge lists to graphs, triangle totals, count persistence and the reference's
// filtered-cost vertex-range partitioner.
#include <stdio.h>
#include <string.h>

#include <cub/cub.cuh>
#include <vector>

#include "accx_internal.h"
#include "devutil.cuh"

__global__ void k_edge_keys(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t k, uint32_t n,
                            unsigned long long *__restrict__ keys, int *__restrict__ bad) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t u = src[i], v = dst[i];
    unsigned long long a = ~0ull, b = ~0ull;  // self loops sort last and are dropped
    if (u >= n || v >= n) {
      atomicOr(bad, 1);
    } else if (u != v) {
      a = ((unsigned long long)u << 32) | v;
      b = ((unsigned long long)v << 32) | u;
    }
    keys[2 * i] = a;
    keys[2 * i + 1] = b;
  }
}

extern "C" int accx_graph_from_edges(const uint32_t *src, const uint32_t *dst, uint64_t k, uint32_t n, void *stream,
                                     accx_graph **out) {
  if (!out || (k && (!src || !dst)) || n == 0) return ACCX_ERR_INVALID_ARG;
  *out = nullptr;
  if (2 * k >= (1ull << 32)) return ACCX_ERR_TOO_LARGE;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return ACCX_ERR_NO_DEVICE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  accx_graph *g = new (std::nothrow) accx_graph();
  if (!g) return ACCX_ERR_OOM;
  cudaGetDevice(&g->device);
  g->symmetric = true;  // both directions of every edge are kept
  unsigned long long *keys = nullptr;
  uint32_t *ds = nullptr, *dd = nullptr;
  int *bad = nullptr, hbad = 0;
  int rc = ACCX_OK;
  do {
    if (cudaMalloc(&keys, sizeof(unsigned long long) * (2 * k + 1)) != cudaSuccess ||
        cudaMalloc(&bad, sizeof(int)) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    const uint32_t *s_src = src, *s_dst = dst;
    if (k && !accx_is_device_ptr(src)) {  // stage host lists
      if (cudaMalloc(&ds, sizeof(uint32_t) * k) != cudaSuccess || cudaMalloc(&dd, sizeof(uint32_t) * k) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
      if (cudaMemcpyAsync(ds, src, sizeof(uint32_t) * k, cudaMemcpyHostToDevice, s) != cudaSuccess ||
          cudaMemcpyAsync(dd, dst, sizeof(uint32_t) * k, cudaMemcpyHostToDevice, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
      s_src = ds;
      s_dst = dd;
    }
    if (cudaMemsetAsync(bad, 0, sizeof(int), s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (k) k_edge_keys<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(s_src, s_dst, k, n, keys, bad);
    if (cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (hbad) { rc = ACCX_ERR_RANGE; break; }
    rc = accx_build_csr_from_keys(g, keys, 2 * k, n, s);
  } while (0);
  if (rc == ACCX_ERR_CUDA || rc == ACCX_ERR_OOM) cudaGetLastError();
  for (void *p : {(void *)keys, (void *)ds, (void *)dd, (void *)bad})
    if (p) cudaFree(p);
  if (rc) {
    accx_graph_free(g);
    return rc;
  }
  *out = g;
  return ACCX_OK;
}

extern "C" int accx_cn_digest(const accx_graph *g, uint64_t *sum, uint64_t *digest, void *stream);

extern "C" int accx_triangles(const accx_graph *g, uint64_t *triangles, void *stream) {
  if (!g || !triangles) return ACCX_ERR_INVALID_ARG;
  uint64_t sum = 0, dig = 0;
  int rc = accx_cn_digest(g, &sum, &dig, stream);
  if (rc) return rc;
  const uint64_t raw = sum - (uint64_t)(int64_t)g->cnt_bias * g->m;
  *triangles = raw / 6;
  return ACCX_OK;
}

struct cn_file_header {
  char magic[8];  // "ACCXCNT1"
  uint32_t n;
  int32_t bias;
  uint64_t m;
};

extern "C" int accx_cn_save(const accx_graph *g, const char *path) {
  if (!g || !path) return ACCX_ERR_INVALID_ARG;
  if (!g->cnt_valid || !g->d_cnt) return ACCX_ERR_NOT_READY;
  std::vector<int32_t> h(g->m);
  if (g->m) ACCX_CUDA_TRY(cudaMemcpy(h.data(), g->d_cnt, sizeof(int32_t) * g->m, cudaMemcpyDeviceToHost));
  FILE *f = fopen(path, "wb");
  if (!f) return ACCX_ERR_IO;
  cn_file_header hd;
  memcpy(hd.magic, "ACCXCNT1", 8);
  hd.n = g->n;
  hd.bias = g->cnt_bias;
  hd.m = g->m;
  bool ok = fwrite(&hd, sizeof(hd), 1, f) == 1 && (g->m == 0 || fwrite(h.data(), 4, g->m, f) == g->m);
  ok = (fclose(f) == 0) && ok;
  return ok ? ACCX_OK : ACCX_ERR_IO;
}

extern "C" int accx_cn_load(accx_graph *g, const char *path) {
  if (!g || !path) return ACCX_ERR_INVALID_ARG;
  FILE *f = fopen(path, "rb");
  if (!f) return ACCX_ERR_IO;
  cn_file_header hd;
  bool ok = fread(&hd, sizeof(hd), 1, f) == 1 && memcmp(hd.magic, "ACCXCNT1", 8) == 0;
  if (!ok || hd.n != g->n || hd.m != g->m) {
    fclose(f);
    return ok ? ACCX_ERR_INVALID_ARG : ACCX_ERR_IO;
  }
  std::vector<int32_t> h(g->m);
  ok = g->m == 0 || fread(h.data(), 4, g->m, f) == g->m;
  fclose(f);
  if (!ok) return ACCX_ERR_IO;
  int rc = accx_ensure_count_scratch(g);
  if (rc) return rc;
  if (g->m) ACCX_CUDA_TRY(cudaMemcpy(g->d_cnt, h.data(), sizeof(int32_t) * g->m, cudaMemcpyHostToDevice));
  g->cnt_bias = hd.bias;
  g->cnt_valid = true;
  g->key_valid.store(false, std::memory_order_release);
  g->qc.query_valid = false;
  g->qc.pairs_valid = false;
  return ACCX_OK;
}

// cost(u) = sum_{v in N(u), v > u} (d_v + 2), a warp per vertex.
__global__ void k_filtered_cost(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst, uint32_t n,
                                unsigned long long *__restrict__ cost) {
  const int lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += nw) {
    unsigned long long c = 0;
    for (uint32_t j = off[u] + lane; j < off[u + 1]; j += 32) {
      const uint32_t v = (uint32_t)dst[j];
      if (v > u) c += off[v + 1] - off[v] + 2;
    }
    for (int d = 16; d >= 1; d >>= 1) c += __shfl_xor_sync(ACCX_FULL_MASK, c, d);
    if (lane == 0) cost[u] = c;
  }
}

extern "C" int accx_vertex_ranges(const accx_graph *g, int parts, uint32_t *ranges, void *stream) {
  if (!g || parts < 1 || !ranges) return ACCX_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t n = g->n;
  unsigned long long *cost = nullptr, *pre = nullptr;
  void *tmp = nullptr;
  size_t tb = 0;
  ACCX_CUDA_TRY(cudaMalloc(&cost, sizeof(unsigned long long) * ((size_t)n + 1)));
  cudaError_t e = cudaMalloc(&pre, sizeof(unsigned long long) * ((size_t)n + 1));
  if (e == cudaSuccess) e = cub::DeviceScan::InclusiveSum(nullptr, tb, cost, pre, (int64_t)n, s);
  if (e == cudaSuccess) e = cudaMalloc(&tmp, tb + 16);
  std::vector<unsigned long long> h((size_t)n + 1, 0);
  if (e == cudaSuccess && n) {
    k_filtered_cost<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(g->d_off, g->d_dst, n, cost);
    e = cub::DeviceScan::InclusiveSum(tmp, tb, cost, pre, (int64_t)n, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data() + 1, pre, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  cudaFree(cost);
  if (pre) cudaFree(pre);
  if (tmp) cudaFree(tmp);
  if (e != cudaSuccess) {
    accx_set_cuda_error(e, "vertex_ranges", __FILE__, __LINE__);
    return ACCX_ERR_CUDA;
  }
  // the reference: ranges[i] = lower_bound(prefix, total / parts * i) over the
  // exclusive prefix array prefix[0..n] (prefix[0] = 0)
  ranges[0] = 0;
  const unsigned long long total = h[n];
  for (int i = 1; i < parts; i++) {
    const unsigned long long target = total / (unsigned long long)parts * (unsigned long long)i;
    ranges[i] = (uint32_t)(std::lower_bound(h.begin(), h.end(), target) - h.begin());
  }
  ranges[parts] = n;
  return ACCX_OK;
}

// Device-side synthetic graph generators and the edge-list -> CSR builder.
//
// The builder does on the GPU what the reference's EdgeListToBinsConverter does
// on the host (scan-query/converter/EdgeListToBinsConverter.cpp:24-126): keep each
// undirected edge once, drop self loops, sort, and emit degrees plus sorted
// adjacency lists.  Unlike the converter it counts degrees after removing
// duplicates, so duplicated input edges cannot produce inconsistent files.
// Sorting and unique-selection use CUB (library code; this is input
// preparation, not the counting path).
#include <cub/cub.cuh>

#include <vector>

#include "accx_internal.h"
#include "gen_host.h"

__global__ void k_gen_keys(int kind, uint64_t seed_mix, uint64_t draws, uint32_t n, int scale,
                           accx_rmat_thresholds t, const uint64_t *__restrict__ cdf,
                           unsigned long long *__restrict__ keys) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < draws; k += stride) {
    uint32_t u, v;
    if (kind == ACCX_GEN_RMAT) accx_rmat_edge(seed_mix, k, scale, t, &u, &v);
    else if (kind == ACCX_GEN_ER) accx_er_edge(seed_mix, k, n, &u, &v);
    else accx_cl_edge(seed_mix, k, cdf, n, &u, &v);
    unsigned long long a = ~0ull, b = ~0ull;  // self loops sort last and are dropped
    if (u != v) {
      a = ((unsigned long long)u << 32) | v;
      b = ((unsigned long long)v << 32) | u;
    }
    keys[2 * k] = a;
    keys[2 * k + 1] = b;
  }
}

// off[w] = first index whose source is >= w; dst = low halves.
__global__ void k_keys_to_csr(const unsigned long long *__restrict__ keys, uint64_t nk, uint32_t n,
                              uint32_t *__restrict__ off, int32_t *__restrict__ dst) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nk; i += stride) {
    int64_t u_prev = (i == 0) ? -1 : (int64_t)(keys[i - 1] >> 32);
    int64_t u_cur = (i == nk) ? (int64_t)n : (int64_t)(keys[i] >> 32);
    for (int64_t w = u_prev + 1; w <= u_cur; w++) off[w] = (uint32_t)i;
    if (i < nk) dst[i] = (int32_t)(keys[i] & 0xffffffffull);
  }
}

int accx_build_csr_from_keys(accx_graph *g, unsigned long long *d_keys, uint64_t nkeys, uint32_t n,
                             cudaStream_t s) {
  // Sort, unique, drop the self-loop sentinel, and fill g->d_off/d_dst.
  unsigned long long *d_alt = nullptr, *d_uniq = nullptr;
  void *d_tmp = nullptr;
  size_t tmp_bytes = 0, tmp2 = 0;
  unsigned long long *d_nsel = nullptr;
  int rc = ACCX_OK;
  do {
    if (accx_dev_alloc((void **)&d_alt, sizeof(unsigned long long) * (nkeys ? nkeys : 1), s) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    cub::DoubleBuffer<unsigned long long> db(d_keys, d_alt);
    if (cub::DeviceRadixSort::SortKeys(nullptr, tmp_bytes, db, (int64_t)nkeys, 0, 64, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (cub::DeviceSelect::Unique(nullptr, tmp2, d_keys, d_alt, d_nsel, (int64_t)nkeys, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (tmp2 > tmp_bytes) tmp_bytes = tmp2;
    if (accx_dev_alloc(&d_tmp, tmp_bytes ? tmp_bytes : 1, s) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    if (accx_dev_alloc((void **)&d_nsel, sizeof(unsigned long long), s) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    if (cub::DeviceRadixSort::SortKeys(d_tmp, tmp_bytes, db, (int64_t)nkeys, 0, 64, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    unsigned long long *sorted = db.Current();
    d_uniq = db.Alternate();
    if (cub::DeviceSelect::Unique(d_tmp, tmp_bytes, sorted, d_uniq, d_nsel, (int64_t)nkeys, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    unsigned long long nu = 0, last = 0;
    if (cudaMemcpyAsync(&nu, d_nsel, sizeof(nu), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (nu) {
      if (cudaMemcpyAsync(&last, d_uniq + nu - 1, sizeof(last), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
      if (last == ~0ull) nu--;
    }
    if (nu >= (1ull << 32) - ACCX_DST_PAD) { rc = ACCX_ERR_TOO_LARGE; break; }
    g->n = n;
    g->m = nu;
    if (accx_dev_alloc((void **)&g->d_off, sizeof(uint32_t) * ((size_t)n + 1), g->home) != cudaSuccess ||
        accx_dev_alloc((void **)&g->d_dst, sizeof(int32_t) * ((size_t)nu + ACCX_DST_PAD), g->home) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    if (cudaMemsetAsync(g->d_dst + nu, 0xff, sizeof(int32_t) * ACCX_DST_PAD, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    int grid = accx_grid_for(g->device, 256, 8);
    k_keys_to_csr<<<grid, 256, 0, s>>>(d_uniq, nu, n, g->d_off, g->d_dst);
    if (cudaGetLastError() != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if ((rc = accx_tilerow_build(g, g->d_off, &g->d_tilerow, s)) != ACCX_OK) break;
    if (cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
  } while (0);
  if (rc == ACCX_ERR_CUDA || rc == ACCX_ERR_OOM) cudaGetLastError();
  accx_dev_free(d_alt, s);
  accx_dev_free(d_tmp, s);
  accx_dev_free(d_nsel, s);
  return rc;
}

extern "C" int accx_graph_generate(const accx_gen_params *p, void *stream, accx_graph **out) {
  if (!p || !out) return ACCX_ERR_INVALID_ARG;
  *out = nullptr;
  uint32_t n;
  uint64_t draws;
  int rc = accx_gen_shape(p, &n, &draws);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return ACCX_ERR_NO_DEVICE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  accx_graph *g = new (std::nothrow) accx_graph();
  if (!g) return ACCX_ERR_OOM;
  cudaGetDevice(&g->device);
  g->home = s;
  g->symmetric = true;  // the edge stream is symmetrised
  unsigned long long *d_keys = nullptr;
  uint64_t *d_cdf = nullptr;
  do {
    if (accx_dev_alloc((void **)&d_keys, sizeof(unsigned long long) * draws * 2, s) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    accx_rmat_thresholds t{};
    if (p->kind == ACCX_GEN_RMAT) t = accx_rmat_make(p->q0, p->q1, p->q2);
    if (p->kind == ACCX_GEN_CHUNG_LU) {
      std::vector<uint64_t> cdf;
      accx_chung_lu_cdf(n, draws, p->q0, p->q1, cdf);
      if (accx_dev_alloc((void **)&d_cdf, sizeof(uint64_t) * cdf.size(), s) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
      if (cudaMemcpyAsync(d_cdf, cdf.data(), sizeof(uint64_t) * cdf.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    }
    int grid = accx_grid_for(g->device, 256, 8);
    k_gen_keys<<<grid, 256, 0, s>>>(p->kind, accx_mix64(p->seed), draws, n, (int)p->p0, t, d_cdf, d_keys);
    if (cudaGetLastError() != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (d_cdf && (cudaStreamSynchronize(s) != cudaSuccess)) { rc = ACCX_ERR_CUDA; break; }
    rc = accx_build_csr_from_keys(g, d_keys, draws * 2, n, s);
  } while (0);
  if (rc == ACCX_ERR_CUDA || rc == ACCX_ERR_OOM) cudaGetLastError();
  accx_dev_free(d_keys, s);
  accx_dev_free(d_cdf, s);
  if (rc) {
    accx_graph_free(g);
    return rc;
  }
  *out = g;
  return ACCX_OK;
}

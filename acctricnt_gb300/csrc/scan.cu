// SCAN structural-clustering query on resident counts.
//
// Reference phases (scan-query-cuda/scan_xp_common.cu): similarity + core check
// (PostComputeCoreChecking :239-267), ClusterCore (:73-85) with the lock-free
// union-find of util/union_find.h:18-35, LabelNonCore/CheckHub (:87-111),
// PostProcess (:113-135), MarkClusterMinEleAsId (:137-158), PrepareResultOutput
// (:160-199) and Graph::Output (util/graph.cu:216-245).
//
// GPU form: one entry-parallel pass decides every similarity bit with the exact
// integer predicate (simpred.h) and counts similar entries per row with
// warp-aggregated atomics (the reference's core_count[u]++ is unsynchronised);
// union-find hooks the larger root under the smaller with atomicCAS, exactly as
// UnionThreadSafe does, so every component's root is its minimum id -- the
// cluster id MarkClusterMinEleAsId assigns; hubs keep the minimum and maximum
// root over core neighbours (two or more distinct roots iff min != max).
#include <cub/cub.cuh>

#include <algorithm>
#include <string>
#include <vector>

#include "accx_internal.h"
#include "devutil.cuh"
#include "simpred.h"

// query counters
#define Q_SIMILAR 0
#define Q_CORES 1
#define Q_CLUSTERS 2
#define Q_HUBS 3
#define Q_OUTLIERS 4
#define Q_PAIRS 5
#define Q_NUM 8

template <int TILE>
__global__ void __launch_bounds__(TILE) k_sim_core(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                                   const int32_t *__restrict__ cnt, uint32_t n, uint32_t m,
                                                   int32_t bias, accx_simq q, uint32_t *__restrict__ simbits,
                                                   int32_t *__restrict__ core_count,
                                                   unsigned long long *__restrict__ qc) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, n, m, base, e, &sh);
  bool sim = false;
  if (e < m) {
    uint32_t v = (uint32_t)dst[e];
    uint32_t du = off[u + 1] - off[u] + 1;
    uint32_t dv = off[v + 1] - off[v] + 1;
    uint32_t cnn = (uint32_t)(cnt[e] - bias + 2);
    sim = accx_similar(q, cnn, du, dv);
  }
  const int lane = threadIdx.x & 31;
  unsigned word = __ballot_sync(ACCX_FULL_MASK, sim);
  if (lane == 0 && base + (threadIdx.x & ~31u) < m) {
    simbits[(base + threadIdx.x) >> 5] = word;
    if (word) atomicAdd(&qc[Q_SIMILAR], (unsigned long long)__popc(word));
  }
  if (sim) {
    unsigned peers = __match_any_sync(word, u);
    if (lane == __ffs(peers) - 1) atomicAdd(&core_count[u], __popc(peers));
  }
}

__global__ void k_label_init(const int32_t *__restrict__ core_count, uint32_t n, int mu, int32_t *__restrict__ label,
                             int32_t *__restrict__ parent, int32_t *__restrict__ hubmin, int32_t *__restrict__ hubmax) {
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    label[u] = core_count[u] >= mu ? ACCX_CORE : ACCX_UNCLASSIFIED;
    parent[u] = (int32_t)u;
    hubmin[u] = 0x7fffffff;
    hubmax[u] = -1;
  }
}

// Root with path halving; parents only ever point to smaller ids.
__device__ __forceinline__ int32_t uf_find(volatile int32_t *parent, int32_t x) {
  int32_t cur = parent[x];
  if (cur != x) {
    int32_t prev = x, next;
    while (cur > (next = parent[cur])) {
      parent[prev] = next;
      prev = cur;
      cur = next;
    }
  }
  return cur;
}

template <int TILE>
__global__ void __launch_bounds__(TILE) k_hook(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                               uint32_t n, uint32_t m, const uint32_t *__restrict__ simbits,
                                               const int32_t *__restrict__ label, int32_t *parent) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, n, m, base, e, &sh);
  if (e >= m) return;
  if (!((simbits[e >> 5] >> (e & 31)) & 1u)) return;
  uint32_t v = (uint32_t)dst[e];
  if (u >= v || label[u] != ACCX_CORE || label[v] != ACCX_CORE) return;
  volatile int32_t *vp = parent;
  // UnionThreadSafe (union_find.h:22-35): hook the larger root under the smaller.
  for (;;) {
    int32_t ru = uf_find(vp, (int32_t)u), rv = uf_find(vp, (int32_t)v);
    if (ru == rv) break;
    int32_t lo = ru < rv ? ru : rv, hi = ru < rv ? rv : ru;
    if (atomicCAS(&parent[hi], hi, lo) == hi) break;
  }
}

__global__ void k_compress(uint32_t n, const int32_t *__restrict__ label, int32_t *parent,
                           unsigned long long *__restrict__ qc) {
  volatile int32_t *vp = parent;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    if (label[u] != ACCX_CORE) continue;
    int32_t r = uf_find(vp, (int32_t)u);
    parent[u] = r;
  }
}

template <int TILE>
__global__ void __launch_bounds__(TILE) k_hub_collect(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                                      uint32_t n, uint32_t m, const int32_t *__restrict__ label,
                                                      const int32_t *__restrict__ parent, int32_t *__restrict__ hubmin,
                                                      int32_t *__restrict__ hubmax) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, n, m, base, e, &sh);
  bool act = false;
  int32_t r = 0;
  if (e < m && label[u] != ACCX_CORE) {
    uint32_t v = (uint32_t)dst[e];
    if (label[v] == ACCX_CORE) {
      act = true;
      r = parent[v];
    }
  }
  unsigned mask = __ballot_sync(ACCX_FULL_MASK, act);
  if (act) {
    unsigned peers = __match_any_sync(mask, u);
    int32_t rmin = __reduce_min_sync(peers, r), rmax = __reduce_max_sync(peers, r);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) {
      atomicMin(&hubmin[u], rmin);
      atomicMax(&hubmax[u], rmax);
    }
  }
}

__global__ void k_finish(uint32_t n, int32_t *__restrict__ label, const int32_t *__restrict__ parent,
                         const int32_t *__restrict__ hubmin, const int32_t *__restrict__ hubmax,
                         int32_t *__restrict__ cluster_out, unsigned long long *__restrict__ qc) {
  unsigned long long cores = 0, clusters = 0, hubs = 0, outl = 0;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    int32_t l = label[u];
    if (l == ACCX_CORE) {
      cores++;
      if (parent[u] == (int32_t)u) clusters++;
    } else if (hubmax[u] >= 0 && hubmin[u] != hubmax[u]) {
      label[u] = ACCX_HUB;
      l = ACCX_HUB;
      hubs++;
    } else {
      outl++;
    }
    if (cluster_out) cluster_out[u] = (l == ACCX_CORE) ? parent[u] : -1;
  }
  cores = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)cores);
  clusters = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)clusters);
  hubs = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)hubs);
  outl = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)outl);
  if ((threadIdx.x & 31) == 0) {
    if (cores) atomicAdd(&qc[Q_CORES], cores);
    if (clusters) atomicAdd(&qc[Q_CLUSTERS], clusters);
    if (hubs) atomicAdd(&qc[Q_HUBS], hubs);
    if (outl) atomicAdd(&qc[Q_OUTLIERS], outl);
  }
}

__global__ void k_bits_to_bytes(const uint32_t *__restrict__ bits, uint32_t m, uint8_t *__restrict__ out) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x)
    out[e] = (bits[e >> 5] >> (e & 31)) & 1u;
}

// (cluster id, non-core vertex) keys for core u, non-core v, similar (u,v).
template <int TILE>
__global__ void __launch_bounds__(TILE) k_pairs(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                                                uint32_t n, uint32_t m, const uint32_t *__restrict__ simbits,
                                                const int32_t *__restrict__ label, const int32_t *__restrict__ parent,
                                                unsigned long long *__restrict__ keys, unsigned long long cap,
                                                unsigned long long *__restrict__ qc) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, n, m, base, e, &sh);
  bool act = false;
  unsigned long long key = 0;
  if (e < m && ((simbits[e >> 5] >> (e & 31)) & 1u) && label[u] == ACCX_CORE) {
    uint32_t v = (uint32_t)dst[e];
    if (label[v] != ACCX_CORE) {
      act = true;
      key = ((unsigned long long)(uint32_t)parent[u] << 32) | v;
    }
  }
  unsigned mask = __ballot_sync(ACCX_FULL_MASK, act);
  if (!mask) return;
  int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
  unsigned long long p = 0;
  if (lane == leader) p = atomicAdd(&qc[Q_PAIRS], (unsigned long long)__popc(mask));
  p = __shfl_sync(ACCX_FULL_MASK, p, leader);
  if (act && keys) {
    unsigned long long idx = p + __popc(mask & ((1u << lane) - 1u));
    if (idx < cap) keys[idx] = key;
  }
}

static int ensure_query_arrays(accx_graph *g) {
  const size_t n = g->n ? g->n : 1, words = (g->m + 31) / 32 + 1;
  if (!g->d_simbits) ACCX_CUDA_TRY(cudaMalloc(&g->d_simbits, sizeof(uint32_t) * words));
  if (!g->d_core_count) ACCX_CUDA_TRY(cudaMalloc(&g->d_core_count, sizeof(int32_t) * n));
  if (!g->d_label) ACCX_CUDA_TRY(cudaMalloc(&g->d_label, sizeof(int32_t) * n));
  if (!g->d_parent) ACCX_CUDA_TRY(cudaMalloc(&g->d_parent, sizeof(int32_t) * n));
  if (!g->d_hubmin) ACCX_CUDA_TRY(cudaMalloc(&g->d_hubmin, sizeof(int32_t) * n));
  if (!g->d_hubmax) ACCX_CUDA_TRY(cudaMalloc(&g->d_hubmax, sizeof(int32_t) * n));
  if (!g->d_qcounters) ACCX_CUDA_TRY(cudaMalloc(&g->d_qcounters, sizeof(unsigned long long) * Q_NUM));
  return ACCX_OK;
}

extern "C" int accx_scan_query(accx_graph *g, double eps, int mu, uint8_t *sim, int32_t *label, int32_t *cluster,
                               accx_scan_summary *summary, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  if (!g->cnt_valid) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  ACCX_CUDA_TRY(cudaSetDevice(g->device));
  int rc = ensure_query_arrays(g);
  if (rc) return rc;
  const uint32_t n = g->n, m = (uint32_t)g->m;
  accx_simq q = accx_simq_make(eps);
  const int sms = accx_sm_count(g->device);
  ACCX_CUDA_TRY(cudaMemsetAsync(g->d_qcounters, 0, sizeof(unsigned long long) * Q_NUM, s));
  ACCX_CUDA_TRY(cudaMemsetAsync(g->d_core_count, 0, sizeof(int32_t) * (n ? n : 1), s));
  const uint32_t tiles = (m + 255) / 256;
  if (m) k_sim_core<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_dst, g->d_cnt, n, m, g->cnt_bias, q, g->d_simbits,
                                               g->d_core_count, g->d_qcounters);
  if (n) k_label_init<<<sms * 4, 256, 0, s>>>(g->d_core_count, n, mu, g->d_label, g->d_parent, g->d_hubmin, g->d_hubmax);
  if (m) k_hook<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_dst, n, m, g->d_simbits, g->d_label, g->d_parent);
  if (n) k_compress<<<sms * 4, 256, 0, s>>>(n, g->d_label, g->d_parent, g->d_qcounters);
  if (m) k_hub_collect<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_dst, n, m, g->d_label, g->d_parent, g->d_hubmin,
                                                  g->d_hubmax);
  bool cl_dev = cluster && accx_is_device_ptr(cluster);
  int32_t *cl_target = cl_dev ? cluster : nullptr;
  if (n) k_finish<<<sms * 4, 256, 0, s>>>(n, g->d_label, g->d_parent, g->d_hubmin, g->d_hubmax, cl_target, g->d_qcounters);
  ACCX_CUDA_TRY(cudaGetLastError());
  g->query_valid = true;
  g->pairs_valid = false;
  g->last_eps = eps;
  g->last_mu = mu;
  if (sim && m) {
    if (accx_is_device_ptr(sim)) {
      k_bits_to_bytes<<<sms * 8, 256, 0, s>>>(g->d_simbits, m, sim);
      ACCX_CUDA_TRY(cudaGetLastError());
    } else {
      uint8_t *tmp = nullptr;
      ACCX_CUDA_TRY(cudaMalloc(&tmp, m));
      k_bits_to_bytes<<<sms * 8, 256, 0, s>>>(g->d_simbits, m, tmp);
      cudaError_t e1 = cudaMemcpyAsync(sim, tmp, m, cudaMemcpyDeviceToHost, s);
      cudaError_t e2 = cudaStreamSynchronize(s);
      cudaFree(tmp);
      if (e1 != cudaSuccess || e2 != cudaSuccess) return ACCX_ERR_CUDA;
    }
  }
  if (label) {
    rc = accx_copy_out(label, g->d_label, sizeof(int32_t) * n, s);
    if (rc) return rc;
  }
  if (cluster && !cl_dev && n) {
    std::vector<int32_t> lab(n), par(n);
    rc = accx_copy_out(lab.data(), g->d_label, sizeof(int32_t) * n, s);
    if (!rc) rc = accx_copy_out(par.data(), g->d_parent, sizeof(int32_t) * n, s);
    if (rc) return rc;
    for (uint32_t u = 0; u < n; u++) cluster[u] = lab[u] == ACCX_CORE ? par[u] : -1;
  }
  unsigned long long h[Q_NUM];
  ACCX_CUDA_TRY(cudaMemcpyAsync(h, g->d_qcounters, sizeof(h), cudaMemcpyDeviceToHost, s));
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  g->summary.cores = (uint32_t)h[Q_CORES];
  g->summary.clusters = (uint32_t)h[Q_CLUSTERS];
  g->summary.hubs = (uint32_t)h[Q_HUBS];
  g->summary.outliers = (uint32_t)h[Q_OUTLIERS];
  g->summary.similar_entries = h[Q_SIMILAR];
  g->summary.noncore_pairs = 0;
  if (summary) *summary = g->summary;
  return ACCX_OK;
}

static int build_pairs(accx_graph *g, cudaStream_t s) {
  if (g->pairs_valid) return ACCX_OK;
  const uint32_t n = g->n, m = (uint32_t)g->m;
  const uint32_t tiles = (m + 255) / 256;
  unsigned long long h = 0;
  ACCX_CUDA_TRY(cudaMemsetAsync(g->d_qcounters + Q_PAIRS, 0, sizeof(unsigned long long), s));
  if (m) k_pairs<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_dst, n, m, g->d_simbits, g->d_label, g->d_parent, nullptr,
                                            0, g->d_qcounters);
  ACCX_CUDA_TRY(cudaMemcpyAsync(&h, g->d_qcounters + Q_PAIRS, sizeof(h), cudaMemcpyDeviceToHost, s));
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  if (h > g->pairs_cap) {
    if (g->d_pairs) cudaFree(g->d_pairs);
    if (g->d_pairs_tmp) cudaFree(g->d_pairs_tmp);
    g->d_pairs = g->d_pairs_tmp = nullptr;
    g->pairs_cap = 0;
    ACCX_CUDA_TRY(cudaMalloc(&g->d_pairs, sizeof(unsigned long long) * h));
    ACCX_CUDA_TRY(cudaMalloc(&g->d_pairs_tmp, sizeof(unsigned long long) * h));
    g->pairs_cap = h;
  }
  g->npairs = 0;
  if (h) {
    ACCX_CUDA_TRY(cudaMemsetAsync(g->d_qcounters + Q_PAIRS, 0, sizeof(unsigned long long), s));
    k_pairs<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_dst, n, m, g->d_simbits, g->d_label, g->d_parent, g->d_pairs,
                                       g->pairs_cap, g->d_qcounters);
    cub::DoubleBuffer<unsigned long long> db(g->d_pairs, g->d_pairs_tmp);
    size_t tb = 0, tb2 = 0;
    unsigned long long *d_nsel = nullptr;
    ACCX_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tb, db, (int64_t)h, 0, 64, s));
    ACCX_CUDA_TRY(cub::DeviceSelect::Unique(nullptr, tb2, g->d_pairs, g->d_pairs_tmp, d_nsel, (int64_t)h, s));
    void *tmp = nullptr;
    ACCX_CUDA_TRY(cudaMalloc(&tmp, std::max(tb, tb2) + 64));
    d_nsel = reinterpret_cast<unsigned long long *>(static_cast<char *>(tmp) + ((std::max(tb, tb2) + 15) & ~size_t(15)));
    cudaError_t e1 = cub::DeviceRadixSort::SortKeys(tmp, tb, db, (int64_t)h, 0, 64, s);
    unsigned long long *sorted = db.Current(), *other = db.Alternate();
    cudaError_t e2 = cub::DeviceSelect::Unique(tmp, tb2, sorted, other, d_nsel, (int64_t)h, s);
    unsigned long long nu = 0;
    cudaError_t e3 = cudaMemcpyAsync(&nu, d_nsel, sizeof(nu), cudaMemcpyDeviceToHost, s);
    cudaError_t e4 = cudaStreamSynchronize(s);
    cudaFree(tmp);
    if (e1 || e2 || e3 || e4) return ACCX_ERR_CUDA;
    if (other != g->d_pairs) std::swap(g->d_pairs, g->d_pairs_tmp);  // unique result lives in d_pairs
    g->npairs = nu;
  }
  g->summary.noncore_pairs = g->npairs;
  g->pairs_valid = true;
  return ACCX_OK;
}

__global__ void k_keys_to_pairs(const unsigned long long *__restrict__ keys, uint64_t np, int32_t *__restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x) {
    out[2 * i] = (int32_t)(keys[i] >> 32);
    out[2 * i + 1] = (int32_t)(keys[i] & 0xffffffffull);
  }
}

extern "C" int accx_scan_pairs(accx_graph *g, int32_t *pairs, uint64_t cap, uint64_t *npairs, void *stream) {
  if (!g || !npairs) return ACCX_ERR_INVALID_ARG;
  if (!g->query_valid) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  ACCX_CUDA_TRY(cudaSetDevice(g->device));
  int rc = build_pairs(g, s);
  if (rc) return rc;
  *npairs = g->npairs;
  if (!pairs) return ACCX_OK;
  if (cap < g->npairs) return ACCX_ERR_TOO_LARGE;
  if (!g->npairs) return ACCX_OK;
  int32_t *tmp = nullptr;
  bool dev = accx_is_device_ptr(pairs);
  if (dev) tmp = pairs; else ACCX_CUDA_TRY(cudaMalloc(&tmp, sizeof(int32_t) * 2 * g->npairs));
  k_keys_to_pairs<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(g->d_pairs, g->npairs, tmp);
  ACCX_CUDA_TRY(cudaGetLastError());
  if (!dev) {
    cudaError_t e1 = cudaMemcpyAsync(pairs, tmp, sizeof(int32_t) * 2 * g->npairs, cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(tmp);
    if (e1 || e2) return ACCX_ERR_CUDA;
  }
  return ACCX_OK;
}

extern "C" int accx_eps_string(double eps, char *out, size_t cap) {
  if (!out || cap == 0) return ACCX_ERR_INVALID_ARG;
  std::string s = std::to_string(eps);
  s.erase(s.find_last_not_of("0u") + 1);
  if (s.size() + 1 > cap) return ACCX_ERR_TOO_LARGE;
  memcpy(out, s.c_str(), s.size() + 1);
  return ACCX_OK;
}

// Decimal writer for the result file (the reference streams ints through an ofstream).
static inline char *put_int(char *p, int32_t v) {
  char tmp[12];
  int k = 0;
  uint32_t x = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
  do { tmp[k++] = (char)('0' + x % 10); x /= 10; } while (x);
  if (v < 0) *p++ = '-';
  while (k) *p++ = tmp[--k];
  return p;
}

extern "C" int accx_write_result(accx_graph *g, const char *dir, double eps, int mu, void *stream) {
  if (!g || !dir) return ACCX_ERR_INVALID_ARG;
  if (!g->query_valid) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  uint64_t np = 0;
  int rc = accx_scan_pairs(g, nullptr, 0, &np, stream);
  if (rc) return rc;
  std::vector<int32_t> pairs(2 * np + 2), lab(g->n + 1), par(g->n + 1);
  rc = accx_scan_pairs(g, pairs.data(), np, &np, stream);
  if (!rc) rc = accx_copy_out(lab.data(), g->d_label, sizeof(int32_t) * g->n, s);
  if (!rc) rc = accx_copy_out(par.data(), g->d_parent, sizeof(int32_t) * g->n, s);
  if (rc) return rc;
  char eps_s[512];
  rc = accx_eps_string(eps, eps_s, sizeof(eps_s));
  if (rc) return rc;
  std::string path = std::string(dir) + "/scanxp-result-" + eps_s + "-" + std::to_string(mu) + ".txt";
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return ACCX_ERR_IO;
  std::vector<char> buf(1 << 22);
  char *p = buf.data(), *lim = buf.data() + buf.size() - 64;
  bool ok = true;
  auto flush = [&]() {
    size_t len = (size_t)(p - buf.data());
    if (len && fwrite(buf.data(), 1, len, f) != len) ok = false;
    p = buf.data();
  };
  const char *hdr = "c/n vertex_id cluster_id\n";
  memcpy(p, hdr, strlen(hdr));
  p += strlen(hdr);
  for (uint32_t i = 0; i < g->n; i++) {
    if (lab[i] != ACCX_CORE) continue;
    *p++ = 'c'; *p++ = ' ';
    p = put_int(p, (int32_t)i);
    *p++ = ' ';
    p = put_int(p, par[i]);
    *p++ = '\n';
    if (p >= lim) flush();
  }
  for (uint64_t k = 0; k < np; k++) {
    *p++ = 'n'; *p++ = ' ';
    p = put_int(p, pairs[2 * k + 1]);
    *p++ = ' ';
    p = put_int(p, pairs[2 * k]);
    *p++ = '\n';
    if (p >= lim) flush();
  }
  flush();
  if (fclose(f) != 0) ok = false;
  return ok ? ACCX_OK : ACCX_ERR_IO;
}

extern "C" int accx_similar_exact(uint32_t cnn, uint32_t du, uint32_t dv, double eps) {
  accx_simq q = accx_simq_make(eps);
  return accx_similar(q, cnn, du, dv) ? 1 : 0;
}

extern "C" int accx_similar_exact_batch(uint64_t k, const uint32_t *cnn, const uint32_t *du, const uint32_t *dv,
                                        double eps, uint8_t *out) {
  if (k && (!cnn || !du || !dv || !out)) return ACCX_ERR_INVALID_ARG;
  accx_simq q = accx_simq_make(eps);
  for (uint64_t i = 0; i < k; i++) out[i] = accx_similar(q, cnn[i], du[i], dv[i]) ? 1 : 0;
  return ACCX_OK;
}

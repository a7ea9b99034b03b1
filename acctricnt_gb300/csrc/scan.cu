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
#include <mutex>
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
#define Q_DIGEST 6
#define Q_BIG 7
#define Q_NUM 8

__device__ __forceinline__ unsigned long long accx_mix64_dev(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Per-entry similarity key, built once after each count: the float nearest to
// x^2 = cnn^2 / (du * dv).  A query compares it with the squared threshold M^2
// of its eps; only keys within 2^-21 (relative) of M^2 -- where float rounding
// could matter -- take the exact-integer test (simpred.h) with cnn, du, dv read
// back from the graph.
template <int TILE>
__global__ void __launch_bounds__(TILE) k_simkey(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow,
                                                 const int32_t *__restrict__ dst, const int32_t *__restrict__ cnt,
                                                 uint32_t n, uint32_t m, int32_t bias, float *__restrict__ key,
                                                 uint32_t *__restrict__ src) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, tilerow, n, m, base, e, &sh);
  if (e >= m) return;
  const uint32_t v = (uint32_t)dst[e];
  const double c = (double)(uint32_t)(cnt[e] - bias + 2);
  const double du = (double)(off[u + 1] - off[u] + 1), dv = (double)(off[v + 1] - off[v] + 1);
  key[e] = (float)(c * c / (du * dv));
  src[e] = u;
}

// Similarity bits from the keys: a streaming pass, one 32-bit word per warp.
__global__ void k_sim_keys(const float *__restrict__ key, const uint32_t *__restrict__ off,
                           const uint32_t *__restrict__ src, const int32_t *__restrict__ dst,
                           const int32_t *__restrict__ cnt, uint32_t n, uint32_t m, int32_t bias, accx_simq q,
                           float lo, float hi, uint32_t *__restrict__ simbits, unsigned long long *__restrict__ qc) {
  const uint32_t stride = gridDim.x * blockDim.x;  // a multiple of 32
  unsigned long long similar = 0;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < ((m + 31) & ~31u); e += stride) {
    bool sim = false;
    if (e < m) {
      if (q.mode != 0) {
        sim = q.mode == 1;
      } else {
        const float k = __ldg(key + e);
        if (k > hi) sim = true;
        else if (k >= lo) {
          // ambiguous band (exact ties x == eps land here): exact test with the
          // entry's own numbers
          const uint32_t u = __ldg(src + e);
          const uint32_t v = (uint32_t)dst[e];
          sim = accx_similar(q, (uint32_t)(cnt[e] - bias + 2), off[u + 1] - off[u] + 1, off[v + 1] - off[v] + 1);
        }
      }
    }
    const unsigned w = __ballot_sync(ACCX_FULL_MASK, sim);
    if ((threadIdx.x & 31) == 0) {
      simbits[e >> 5] = w;
      similar += __popc(w);
    }
  }
  if ((threadIdx.x & 31) == 0 && similar) atomicAdd(&qc[Q_SIMILAR], similar);
}

// Cores from the similarity bits: core_count[u] = popcount of row u's bits.
// One thread per vertex; rows longer than BIG_ROW are left to k_cores_big (one
// CTA each).  Also resets labels, union-find roots, hub ranges and writes the
// core bitmap (n/8 bytes, kept in L2 for the random lookups that follow).
#define BIG_ROW 4096
__device__ __forceinline__ uint32_t accx_row_popc(const uint32_t *__restrict__ bits, uint32_t b, uint32_t e) {
  uint32_t c = 0;
  if (b >= e) return 0;
  const uint32_t w0 = b >> 5, w1 = (e - 1) >> 5;
  for (uint32_t w = w0; w <= w1; w++) {
    uint32_t x = __ldg(bits + w);
    if (w == w0) x &= 0xffffffffu << (b & 31);
    if (w == w1 && (e & 31)) x &= 0xffffffffu >> (32 - (e & 31));
    c += __popc(x);
  }
  return c;
}

__global__ void k_cores(const uint32_t *__restrict__ off, uint32_t n, int mu, const uint32_t *__restrict__ simbits,
                        int32_t *__restrict__ core_count, int32_t *__restrict__ label, int32_t *__restrict__ parent,
                        int32_t *__restrict__ hubmin, int32_t *__restrict__ hubmax, uint32_t *__restrict__ corebits,
                        uint32_t *__restrict__ big, unsigned long long *__restrict__ qc) {
  const uint32_t stride = gridDim.x * blockDim.x;  // a multiple of 32
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < ((n + 31) & ~31u); u += stride) {
    bool core = false;
    if (u < n) {
      const uint32_t b = off[u], e = off[u + 1];
      if (e - b > BIG_ROW) {
        const unsigned long long p = atomicAdd(&qc[Q_BIG], 1ull);
        big[p] = u;  // counted by k_cores_big
      } else {
        const uint32_t c = accx_row_popc(simbits, b, e);
        core_count[u] = (int32_t)c;
        core = (int)c >= mu;
        label[u] = core ? ACCX_CORE : ACCX_UNCLASSIFIED;
      }
      parent[u] = (int32_t)u;
      hubmin[u] = 0x7fffffff;
      hubmax[u] = -1;
    }
    const unsigned w = __ballot_sync(ACCX_FULL_MASK, core);
    if ((threadIdx.x & 31) == 0 && u < n) corebits[u >> 5] = w;
  }
}

__global__ void __launch_bounds__(256) k_cores_big(const uint32_t *__restrict__ off, int mu,
                                                   const uint32_t *__restrict__ simbits, const uint32_t *__restrict__ big,
                                                   const unsigned long long *__restrict__ qc,
                                                   int32_t *__restrict__ core_count, int32_t *__restrict__ label,
                                                   uint32_t *__restrict__ corebits) {
  __shared__ uint32_t part[8];
  const unsigned long long nb = qc[Q_BIG];
  for (unsigned long long i = blockIdx.x; i < nb; i += gridDim.x) {
    const uint32_t u = big[i], b = off[u], e = off[u + 1];
    uint32_t c = 0;
    const uint32_t w0 = b >> 5, w1 = (e - 1) >> 5;
    for (uint32_t w = w0 + threadIdx.x; w <= w1; w += blockDim.x) {
      uint32_t x = __ldg(simbits + w);
      if (w == w0) x &= 0xffffffffu << (b & 31);
      if (w == w1 && (e & 31)) x &= 0xffffffffu >> (32 - (e & 31));
      c += __popc(x);
    }
    c = __reduce_add_sync(ACCX_FULL_MASK, c);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += part[k];
      core_count[u] = (int32_t)t;
      const bool core = (int)t >= mu;
      label[u] = core ? ACCX_CORE : ACCX_UNCLASSIFIED;
      if (core) atomicOr(&corebits[u >> 5], 1u << (u & 31));
    }
    __syncthreads();
  }
}

__device__ __forceinline__ bool accx_is_core(const uint32_t *__restrict__ corebits, uint32_t v) {
  return (__ldg(corebits + (v >> 5)) >> (v & 31)) & 1u;
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

// Union over similar core-core entries: one thread per similarity word, only
// set bits do work.  UnionThreadSafe (union_find.h:22-35): hook the larger root
// under the smaller.
__global__ void k_hook_words(const uint32_t *__restrict__ src, const int32_t *__restrict__ dst, uint32_t m,
                             const uint32_t *__restrict__ simbits,
                             const uint32_t *__restrict__ corebits, int32_t *parent) {
  volatile int32_t *vp = parent;
  const uint32_t words = (m + 31) / 32;
  for (uint32_t wi = blockIdx.x * blockDim.x + threadIdx.x; wi < words; wi += gridDim.x * blockDim.x) {
    uint32_t w = __ldg(simbits + wi);
    while (w) {
      const uint32_t e = wi * 32u + (uint32_t)(__ffs(w) - 1);
      w &= w - 1;
      const uint32_t v = (uint32_t)dst[e];
      if (!accx_is_core(corebits, v)) continue;
      const uint32_t u = __ldg(src + e);
      if (u >= v || !accx_is_core(corebits, u)) continue;
      for (;;) {
        int32_t ru = uf_find(vp, (int32_t)u), rv = uf_find(vp, (int32_t)v);
        if (ru == rv) break;
        int32_t lo = ru < rv ? ru : rv, hi = ru < rv ? rv : ru;
        if (atomicCAS(&parent[hi], hi, lo) == hi) break;
      }
    }
  }
}

__global__ void k_compress(uint32_t n, const uint32_t *__restrict__ corebits, int32_t *parent) {
  volatile int32_t *vp = parent;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    if (!accx_is_core(corebits, u)) continue;
    parent[u] = uf_find(vp, (int32_t)u);
  }
}

// Hubs, pushed from the core side: a warp per core vertex v streams N(v) and
// folds v's cluster root into the [min, max] range of every non-core neighbour
// (CheckHub ignores similarity: any core neighbour counts).
__global__ void k_hub_push(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst, uint32_t n,
                           const uint32_t *__restrict__ corebits, const int32_t *__restrict__ parent,
                           int32_t *__restrict__ hubmin, int32_t *__restrict__ hubmax) {
  const int lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  const uint32_t words = (n + 31) / 32;
  for (uint32_t wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < words; wi += nw) {
    uint32_t cw = __ldg(corebits + wi);
    while (cw) {
      const uint32_t v = wi * 32u + (uint32_t)(__ffs(cw) - 1);
      cw &= cw - 1;
      const uint32_t b = off[v], e = off[v + 1];
      if (e - b > BIG_ROW) continue;  // k_hub_push_big spreads long rows over many CTAs
      const int32_t r = parent[v];
      for (uint32_t j = b + lane; j < e; j += 32) {
        const uint32_t u = (uint32_t)dst[j];
        if (accx_is_core(corebits, u)) continue;
        atomicMin(&hubmin[u], r);
        atomicMax(&hubmax[u], r);
      }
    }
  }
}

// The long core rows (the big list of k_cores): blockIdx.y walks the list,
// blockIdx.x and the threads split each row.
__global__ void k_hub_push_big(const uint32_t *__restrict__ off, const int32_t *__restrict__ dst,
                               const uint32_t *__restrict__ big, const unsigned long long *__restrict__ qc,
                               const uint32_t *__restrict__ corebits, const int32_t *__restrict__ parent,
                               int32_t *__restrict__ hubmin, int32_t *__restrict__ hubmax) {
  const unsigned long long nb = qc[Q_BIG];
  for (unsigned long long i = blockIdx.y; i < nb; i += gridDim.y) {
    const uint32_t v = big[i];
    if (!accx_is_core(corebits, v)) continue;
    const int32_t r = parent[v];
    const uint32_t b = off[v], e = off[v + 1];
    for (uint32_t j = b + blockIdx.x * blockDim.x + threadIdx.x; j < e; j += gridDim.x * blockDim.x) {
      const uint32_t u = (uint32_t)dst[j];
      if (accx_is_core(corebits, u)) continue;
      atomicMin(&hubmin[u], r);
      atomicMax(&hubmax[u], r);
    }
  }
}

__global__ void k_finish(uint32_t n, int32_t *__restrict__ label, const int32_t *__restrict__ parent,
                         const int32_t *__restrict__ hubmin, const int32_t *__restrict__ hubmax,
                         int32_t *__restrict__ cluster_out, unsigned long long *__restrict__ qc) {
  unsigned long long cores = 0, clusters = 0, hubs = 0, outl = 0, dig = 0;
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
    const int32_t cl = (l == ACCX_CORE) ? parent[u] : -1;
    if (cluster_out) cluster_out[u] = cl;
    dig += accx_mix64_dev(((unsigned long long)u << 34) ^ ((unsigned long long)(uint32_t)l << 32) ^ (uint32_t)cl);
  }
  cores = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)cores);
  clusters = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)clusters);
  hubs = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)hubs);
  outl = __reduce_add_sync(ACCX_FULL_MASK, (unsigned)outl);
  for (int d = 16; d >= 1; d >>= 1) dig += __shfl_xor_sync(ACCX_FULL_MASK, dig, d);
  if ((threadIdx.x & 31) == 0) {
    if (dig) atomicAdd(&qc[Q_DIGEST], dig);
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
__global__ void __launch_bounds__(TILE) k_pairs(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow, const int32_t *__restrict__ dst,
                                                uint32_t n, uint32_t m, const uint32_t *__restrict__ simbits,
                                                const int32_t *__restrict__ label, const int32_t *__restrict__ parent,
                                                unsigned long long *__restrict__ keys, unsigned long long cap,
                                                unsigned long long *__restrict__ qc) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, tilerow, n, m, base, e, &sh);
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

void accx_query_ctx_release(accx_query_ctx *q) {
  void *ptrs[] = {q->d_simbits, q->d_core_count, q->d_label,     q->d_parent, q->d_hubmin,
                  q->d_hubmax,  q->d_qcounters,  q->d_pairs,     q->d_pairs_tmp, q->d_corebits, q->d_big};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  *q = accx_query_ctx();
}

static int ensure_query_arrays(const accx_graph *g, accx_query_ctx *q) {
  if (q->d_simbits && (q->n != g->n || q->m != g->m)) return ACCX_ERR_INVALID_ARG;  // made for another graph
  q->n = g->n;
  q->m = g->m;
  const size_t n = g->n ? g->n : 1, words = (g->m + 31) / 32 + 1;
  if (!q->d_simbits) ACCX_CUDA_TRY(cudaMalloc(&q->d_simbits, sizeof(uint32_t) * words));
  if (!q->d_core_count) ACCX_CUDA_TRY(cudaMalloc(&q->d_core_count, sizeof(int32_t) * n));
  if (!q->d_label) ACCX_CUDA_TRY(cudaMalloc(&q->d_label, sizeof(int32_t) * n));
  if (!q->d_parent) ACCX_CUDA_TRY(cudaMalloc(&q->d_parent, sizeof(int32_t) * n));
  if (!q->d_hubmin) ACCX_CUDA_TRY(cudaMalloc(&q->d_hubmin, sizeof(int32_t) * n));
  if (!q->d_hubmax) ACCX_CUDA_TRY(cudaMalloc(&q->d_hubmax, sizeof(int32_t) * n));
  if (!q->d_qcounters) ACCX_CUDA_TRY(cudaMalloc(&q->d_qcounters, sizeof(unsigned long long) * Q_NUM));
  if (!q->d_corebits) ACCX_CUDA_TRY(cudaMalloc(&q->d_corebits, sizeof(uint32_t) * (n / 32 + 2)));
  if (!q->d_big) ACCX_CUDA_TRY(cudaMalloc(&q->d_big, sizeof(uint32_t) * (g->m / BIG_ROW + 2)));
  return ACCX_OK;
}

extern "C" int accx_scan_query_ctx(const accx_graph *g, accx_query_ctx *q, double eps, int mu, uint8_t *sim,
                                   int32_t *label, int32_t *cluster, accx_scan_summary *summary, void *stream) {
  if (!g || !q) return ACCX_ERR_INVALID_ARG;
  if (!g->cnt_valid) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  ACCX_CUDA_TRY(cudaSetDevice(g->device));
  int rc = ensure_query_arrays(g, q);
  if (rc) return rc;
  const uint32_t n = g->n, m = (uint32_t)g->m;
  const accx_simq sq = accx_simq_make(eps);
  const int sms = accx_sm_count(g->device);
  ACCX_CUDA_TRY(cudaMemsetAsync(q->d_qcounters, 0, sizeof(unsigned long long) * Q_NUM, s));
  const uint32_t tiles = (m + 255) / 256;
  if (m && !g->key_valid.load(std::memory_order_acquire)) {
    // once per count; several threads may query one const handle, so the key
    // array is built under a lock
    static std::mutex mu_key;
    std::lock_guard<std::mutex> lk(mu_key);
    if (!g->key_valid.load(std::memory_order_relaxed)) {
      accx_graph *gm = const_cast<accx_graph *>(g);
      if (!gm->d_simkey) {
        ACCX_CUDA_TRY(accx_dev_alloc((void **)&gm->d_simkey, sizeof(float) * (size_t)m, g->home));
        ACCX_CUDA_TRY(accx_dev_alloc((void **)&gm->d_src, sizeof(uint32_t) * (size_t)m, g->home));
        if (g->home) ACCX_CUDA_TRY(cudaStreamSynchronize(g->home));
      }
      k_simkey<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_tilerow, g->d_dst, g->d_cnt, n, m, g->cnt_bias, gm->d_simkey,
                                          gm->d_src);
      ACCX_CUDA_TRY(cudaStreamSynchronize(s));
      gm->key_valid.store(true, std::memory_order_release);
    }
  }
  // threshold band on the keys: exact outside, simpred.h inside
  const float klo = sq.mode == 0 ? (float)sq.m2_lo * (1.0f - 4e-7f) : 0.f;
  const float khi = sq.mode == 0 ? (float)sq.m2_hi * (1.0f + 4e-7f) : 0.f;
  if (m) k_sim_keys<<<sms * 8, 256, 0, s>>>(g->d_simkey, g->d_off, g->d_src, g->d_dst, g->d_cnt, n, m, g->cnt_bias,
                                            sq, klo, khi, q->d_simbits, q->d_qcounters);
  if (n) {
    k_cores<<<sms * 8, 256, 0, s>>>(g->d_off, n, mu, q->d_simbits, q->d_core_count, q->d_label, q->d_parent,
                                    q->d_hubmin, q->d_hubmax, q->d_corebits, q->d_big, q->d_qcounters);
    k_cores_big<<<sms * 2, 256, 0, s>>>(g->d_off, mu, q->d_simbits, q->d_big, q->d_qcounters, q->d_core_count,
                                        q->d_label, q->d_corebits);
  }
  if (m) k_hook_words<<<sms * 8, 256, 0, s>>>(g->d_src, g->d_dst, m, q->d_simbits, q->d_corebits, q->d_parent);
  if (n) k_compress<<<sms * 4, 256, 0, s>>>(n, q->d_corebits, q->d_parent);
  if (n) {
    k_hub_push<<<sms * 8, 256, 0, s>>>(g->d_off, g->d_dst, n, q->d_corebits, q->d_parent, q->d_hubmin, q->d_hubmax);
    k_hub_push_big<<<dim3(16, 64), 256, 0, s>>>(g->d_off, g->d_dst, q->d_big, q->d_qcounters, q->d_corebits,
                                                 q->d_parent, q->d_hubmin, q->d_hubmax);
  }
  bool cl_dev = cluster && accx_is_device_ptr(cluster);
  int32_t *cl_target = cl_dev ? cluster : nullptr;
  if (n) k_finish<<<sms * 4, 256, 0, s>>>(n, q->d_label, q->d_parent, q->d_hubmin, q->d_hubmax, cl_target, q->d_qcounters);
  ACCX_CUDA_TRY(cudaGetLastError());
  q->query_valid = true;
  q->pairs_valid = false;
  q->last_eps = eps;
  q->last_mu = mu;
  if (sim && m) {
    if (accx_is_device_ptr(sim)) {
      k_bits_to_bytes<<<sms * 8, 256, 0, s>>>(q->d_simbits, m, sim);
      ACCX_CUDA_TRY(cudaGetLastError());
    } else {
      uint8_t *tmp = nullptr;
      ACCX_CUDA_TRY(cudaMalloc(&tmp, m));
      k_bits_to_bytes<<<sms * 8, 256, 0, s>>>(q->d_simbits, m, tmp);
      cudaError_t e1 = cudaMemcpyAsync(sim, tmp, m, cudaMemcpyDeviceToHost, s);
      cudaError_t e2 = cudaStreamSynchronize(s);
      cudaFree(tmp);
      if (e1 != cudaSuccess || e2 != cudaSuccess) return ACCX_ERR_CUDA;
    }
  }
  if (label) {
    rc = accx_copy_out(label, q->d_label, sizeof(int32_t) * n, s);
    if (rc) return rc;
  }
  if (cluster && !cl_dev && n) {
    std::vector<int32_t> lab(n), par(n);
    rc = accx_copy_out(lab.data(), q->d_label, sizeof(int32_t) * n, s);
    if (!rc) rc = accx_copy_out(par.data(), q->d_parent, sizeof(int32_t) * n, s);
    if (rc) return rc;
    for (uint32_t u = 0; u < n; u++) cluster[u] = lab[u] == ACCX_CORE ? par[u] : -1;
  }
  unsigned long long h[Q_NUM];
  ACCX_CUDA_TRY(cudaMemcpyAsync(h, q->d_qcounters, sizeof(h), cudaMemcpyDeviceToHost, s));
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  q->summary.cores = (uint32_t)h[Q_CORES];
  q->summary.clusters = (uint32_t)h[Q_CLUSTERS];
  q->summary.hubs = (uint32_t)h[Q_HUBS];
  q->summary.outliers = (uint32_t)h[Q_OUTLIERS];
  q->summary.similar_entries = h[Q_SIMILAR];
  q->summary.digest = h[Q_DIGEST];
  q->summary.noncore_pairs = 0;
  if (summary) *summary = q->summary;
  return ACCX_OK;
}

extern "C" int accx_scan_query(accx_graph *g, double eps, int mu, uint8_t *sim, int32_t *label, int32_t *cluster,
                               accx_scan_summary *summary, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  return accx_scan_query_ctx(g, &g->qc, eps, mu, sim, label, cluster, summary, stream);
}

extern "C" int accx_query_ctx_create(const accx_graph *g, accx_query_ctx **out) {
  if (!g || !out) return ACCX_ERR_INVALID_ARG;
  accx_query_ctx *q = new (std::nothrow) accx_query_ctx();
  if (!q) return ACCX_ERR_OOM;
  int rc = ensure_query_arrays(g, q);
  if (rc) {
    accx_query_ctx_release(q);
    delete q;
    return rc;
  }
  *out = q;
  return ACCX_OK;
}

extern "C" int accx_query_ctx_free(accx_query_ctx *q) {
  if (!q) return ACCX_ERR_INVALID_ARG;
  accx_query_ctx_release(q);
  delete q;
  return ACCX_OK;
}

static int build_pairs(accx_graph *g, accx_query_ctx *q, cudaStream_t s) {
  if (q->pairs_valid) return ACCX_OK;
  const uint32_t n = g->n, m = (uint32_t)g->m;
  const uint32_t tiles = (m + 255) / 256;
  unsigned long long h = 0;
  ACCX_CUDA_TRY(cudaMemsetAsync(q->d_qcounters + Q_PAIRS, 0, sizeof(unsigned long long), s));
  if (m) k_pairs<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_tilerow, g->d_dst, n, m, q->d_simbits, q->d_label, q->d_parent, nullptr,
                                            0, q->d_qcounters);
  ACCX_CUDA_TRY(cudaMemcpyAsync(&h, q->d_qcounters + Q_PAIRS, sizeof(h), cudaMemcpyDeviceToHost, s));
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  if (h > q->pairs_cap) {
    if (q->d_pairs) cudaFree(q->d_pairs);
    if (q->d_pairs_tmp) cudaFree(q->d_pairs_tmp);
    q->d_pairs = q->d_pairs_tmp = nullptr;
    q->pairs_cap = 0;
    ACCX_CUDA_TRY(cudaMalloc(&q->d_pairs, sizeof(unsigned long long) * h));
    ACCX_CUDA_TRY(cudaMalloc(&q->d_pairs_tmp, sizeof(unsigned long long) * h));
    q->pairs_cap = h;
  }
  q->npairs = 0;
  if (h) {
    ACCX_CUDA_TRY(cudaMemsetAsync(q->d_qcounters + Q_PAIRS, 0, sizeof(unsigned long long), s));
    k_pairs<256><<<tiles, 256, 0, s>>>(g->d_off, g->d_tilerow, g->d_dst, n, m, q->d_simbits, q->d_label, q->d_parent, q->d_pairs,
                                       q->pairs_cap, q->d_qcounters);
    cub::DoubleBuffer<unsigned long long> db(q->d_pairs, q->d_pairs_tmp);
    size_t tb = 0, tb2 = 0;
    unsigned long long *d_nsel = nullptr;
    ACCX_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tb, db, (int64_t)h, 0, 64, s));
    ACCX_CUDA_TRY(cub::DeviceSelect::Unique(nullptr, tb2, q->d_pairs, q->d_pairs_tmp, d_nsel, (int64_t)h, s));
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
    if (other != q->d_pairs) std::swap(q->d_pairs, q->d_pairs_tmp);  // unique result lives in d_pairs
    q->npairs = nu;
  }
  q->summary.noncore_pairs = q->npairs;
  q->pairs_valid = true;
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
  if (!g->qc.query_valid) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  ACCX_CUDA_TRY(cudaSetDevice(g->device));
  accx_query_ctx *q = &g->qc;
  int rc = build_pairs(g, q, s);
  if (rc) return rc;
  *npairs = q->npairs;
  if (!pairs) return ACCX_OK;
  if (cap < q->npairs) return ACCX_ERR_TOO_LARGE;
  if (!q->npairs) return ACCX_OK;
  int32_t *tmp = nullptr;
  bool dev = accx_is_device_ptr(pairs);
  if (dev) tmp = pairs; else ACCX_CUDA_TRY(cudaMalloc(&tmp, sizeof(int32_t) * 2 * q->npairs));
  k_keys_to_pairs<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(q->d_pairs, q->npairs, tmp);
  ACCX_CUDA_TRY(cudaGetLastError());
  if (!dev) {
    cudaError_t e1 = cudaMemcpyAsync(pairs, tmp, sizeof(int32_t) * 2 * q->npairs, cudaMemcpyDeviceToHost, s);
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
  accx_query_ctx *q = &g->qc;
  if (!q->query_valid) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  uint64_t np = 0;
  int rc = accx_scan_pairs(g, nullptr, 0, &np, stream);
  if (rc) return rc;
  std::vector<int32_t> pairs(2 * np + 2), lab(g->n + 1), par(g->n + 1);
  rc = accx_scan_pairs(g, pairs.data(), np, &np, stream);
  if (!rc) rc = accx_copy_out(lab.data(), q->d_label, sizeof(int32_t) * g->n, s);
  if (!rc) rc = accx_copy_out(par.data(), q->d_parent, sizeof(int32_t) * g->n, s);
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

__global__ void k_cnt_digest(const int32_t *__restrict__ cnt, uint32_t m, unsigned long long *__restrict__ out) {
  unsigned long long sum = 0, dig = 0;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
    const uint32_t c = (uint32_t)cnt[e];
    sum += c;
    dig += accx_mix64_dev(((unsigned long long)e << 32) | c);
  }
  for (int d = 16; d >= 1; d >>= 1) {
    sum += __shfl_xor_sync(ACCX_FULL_MASK, sum, d);
    dig += __shfl_xor_sync(ACCX_FULL_MASK, dig, d);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out[0], sum);
    atomicAdd(&out[1], dig);
  }
}

extern "C" int accx_cn_digest(const accx_graph *g, uint64_t *sum, uint64_t *digest, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  if (!g->cnt_valid) return ACCX_ERR_NOT_READY;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long *d = nullptr, h[2] = {0, 0};
  ACCX_CUDA_TRY(accx_dev_alloc((void **)&d, sizeof(h), s));
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(h), s);
  if (e == cudaSuccess && g->m) {
    k_cnt_digest<<<accx_sm_count(g->device) * 4, 256, 0, s>>>(g->d_cnt, (uint32_t)g->m, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  accx_dev_free(d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    accx_set_cuda_error(e, "cn_digest", __FILE__, __LINE__);
    return ACCX_ERR_CUDA;
  }
  if (sum) *sum = h[0];
  if (digest) *digest = h[1];
  return ACCX_OK;
}

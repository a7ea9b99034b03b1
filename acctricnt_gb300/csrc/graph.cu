// Graph handles: upload, file loading, validation, download; status strings.
//
// Replaces the reference's Graph loader (scan-query-cuda/util/graph.cu:33-214):
// the same b_degree.bin / b_adj.bin format and the same input checks
// (CheckInputGraph: no self loops, strictly increasing rows), plus a range and a
// symmetry check the reference leaves implicit, run as one GPU pass.  Arrays live
// in plain device memory for the handle's lifetime instead of managed memory.
#include <errno.h>
#include <stdlib.h>
#include <string.h>

#include <cub/cub.cuh>

#include <mutex>
#include <string>
#include <vector>

#include "accx_internal.h"
#include "devutil.cuh"

static thread_local char g_last_cuda_error[512];

void accx_set_cuda_error(cudaError_t e, const char *what, const char *file, int line) {
  snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "%s at %s:%d: %s", cudaGetErrorString(e), file, line,
           what);
  if (getenv("ACCX_DEBUG")) fprintf(stderr, "[accx] CUDA error %s\n", g_last_cuda_error);
}

extern "C" const char *accx_strerror(int status) {
  switch (status) {
    case ACCX_OK: return "ok";
    case ACCX_ERR_INVALID_ARG: return "invalid argument";
    case ACCX_ERR_CUDA: return g_last_cuda_error[0] ? g_last_cuda_error : "CUDA error";
    case ACCX_ERR_OOM: return "out of memory";
    case ACCX_ERR_SELF_LOOP: return "Self loop";
    case ACCX_ERR_UNSORTED: return "Edges not sorted in increasing id order!";
    case ACCX_ERR_RANGE: return "neighbour id or offsets out of range";
    case ACCX_ERR_ASYMMETRIC: return "graph is not symmetric";
    case ACCX_ERR_IO: return "file cannot be read or written";
    case ACCX_ERR_TOO_LARGE: return "size beyond the supported maximum";
    case ACCX_ERR_NOT_READY: return "not ready";
    case ACCX_ERR_TIMEOUT: return "bounded device wait timed out";
    case ACCX_ERR_ADMISSION: return "request exceeds the HBM budget";
    case ACCX_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

extern "C" const char *accx_version(void) { return ACCX_VERSION_STR; }

// Device memory comes from the device's default stream-ordered pool, whose
// release threshold is raised once per device so that freed blocks stay cached
// for the next graph (creating and freeing graphs of the same size then costs no
// page mapping).  cudaMemPoolTrimTo on cudaDeviceGetDefaultMemPool returns them.
static void accx_pool_setup() {
  static std::once_flag once[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return;
  }
  std::call_once(once[dev], [dev] {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  });
}

// With a stream: ordered on it.  Without: ordered on the legacy stream and
// waited for, so the block is usable from any stream on return.
cudaError_t accx_dev_alloc(void **p, size_t bytes, cudaStream_t s) {
  accx_pool_setup();
  if (s) return cudaMallocAsync(p, bytes, s);
  cudaError_t e = cudaMallocAsync(p, bytes, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  return e;
}

// Without a stream the device is synchronised first, as cudaFree does: work on
// any stream may still read the block.
void accx_dev_free(void *p, cudaStream_t s) {
  if (!p) return;
  if (s) {
    cudaFreeAsync(p, s);
  } else {
    cudaDeviceSynchronize();
    cudaFreeAsync(p, 0);
  }
}

bool accx_is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Host <-> device copies.  Pinned host memory is mapped into the GPU's address
// space; on GB300 with its coherent host link a copy kernel moves it through
// that mapping at link speed, where the copy engines were measured several
// times slower into device blocks that had been freed and reused.  Pageable
// host memory and unaligned ends go through cudaMemcpyAsync.
// Each thread keeps four 16-byte loads in flight (each warp still reads 512
// contiguous bytes per load): the host link's latency is long.
__global__ void k_copy16(uint4 *__restrict__ d, const uint4 *__restrict__ s, size_t n16) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
    d[i] = a;
    d[i + stride] = b;
    d[i + 2 * stride] = c;
    d[i + 3 * stride] = e;
  }
  for (; i < n16; i += stride) d[i] = s[i];
}

// The device-side address of pinned (mapped) host memory, or nullptr.
static void *mapped_host(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void *accx_mapped_host(const void *p) { return mapped_host(p); }

static cudaError_t copy_via_kernel(void *d, const void *sp, size_t bytes, cudaStream_t s) {
  const size_t n16 = bytes / 16, head = n16 * 16;
  if (n16) {
    int dev = 0;
    cudaGetDevice(&dev);
    k_copy16<<<accx_sm_count(dev) * 8, 256, 0, s>>>(static_cast<uint4 *>(d), static_cast<const uint4 *>(sp), n16);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (bytes > head)
    return cudaMemcpyAsync(static_cast<char *>(d) + head, static_cast<const char *>(sp) + head, bytes - head,
                           cudaMemcpyDefault, s);
  return cudaSuccess;
}

int accx_copy_out(void *dst, const void *dev_src, size_t bytes, cudaStream_t s) {
  if (!bytes) return ACCX_OK;
  if (accx_is_device_ptr(dst)) {
    ACCX_CUDA_TRY(cudaMemcpyAsync(dst, dev_src, bytes, cudaMemcpyDefault, s));
    return ACCX_OK;
  }
  void *m = mapped_host(dst);
  if (m && !(((uintptr_t)m | (uintptr_t)dev_src) & 15)) ACCX_CUDA_TRY(copy_via_kernel(m, dev_src, bytes, s));
  else ACCX_CUDA_TRY(cudaMemcpyAsync(dst, dev_src, bytes, cudaMemcpyDefault, s));
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  return ACCX_OK;
}

int accx_copy_in(void *dev_dst, const void *src, size_t bytes, cudaStream_t s) {
  if (!bytes) return ACCX_OK;
  if (accx_is_device_ptr(src)) {
    ACCX_CUDA_TRY(cudaMemcpyAsync(dev_dst, src, bytes, cudaMemcpyDefault, s));
    return ACCX_OK;
  }
  const void *m = mapped_host(src);
  if (m && !(((uintptr_t)m | (uintptr_t)dev_dst) & 15)) ACCX_CUDA_TRY(copy_via_kernel(dev_dst, m, bytes, s));
  else ACCX_CUDA_TRY(cudaMemcpyAsync(dev_dst, src, bytes, cudaMemcpyDefault, s));
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  return ACCX_OK;
}

int accx_sm_count(int device) {
  static int cached[64] = {0};
  if (device < 0 || device >= 64) return 1;
  if (!cached[device]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0) v = 1;
    cached[device] = v;
  }
  return cached[device];
}

int accx_grid_for(int device, int block, int per_sm) {
  (void)block;
  return accx_sm_count(device) * per_sm;
}

// ---------------------------------------------------------------------------
// Validation: one thread per entry sets a bit per kind of defect; the host
// reports them in the reference's order (range, self loop, order), then symmetry.
#define V_RANGE 1
#define V_SELF 2
#define V_UNSORTED 4
#define V_ASYM 8
// Range checks always run (every kernel indexes off[] with neighbour ids); the
// order and self-loop checks run when `full` is set.  Symmetry is checked after
// this pass by sorting the entries by neighbour id (k_rev_check).  SEARCH: the
// fallback when the sort's buffers do not fit, a search per entry pair -- of the
// two entries of a pair only the one whose target has the smaller degree (ties:
// the larger target id) searches its reverse, in that shorter list, and the
// searching entries are counted.  If every searching entry finds its reverse (a
// non-searching entry; distinct entries have distinct reverses in sorted lists
// without repeats) and they are exactly half of all entries, the reverse map is a
// bijection onto the other half: the graph is symmetric.
// Symmetry fingerprints: two published 64-bit finalisers (SplitMix64's, and
// MurmurHash3's fmix64 applied to the key plus an odd constant) of the key
// (a << 32 | b).  Over all entries, sum of f(u,v) - f(v,u) is zero (mod 2^64) on
// a symmetric graph.
__device__ __forceinline__ unsigned long long fp_splitmix(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ unsigned long long fp_fmix(unsigned long long k) {
  k += 0x9e3779b97f4a7c15ull;
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  return k ^ (k >> 33);
}
#define FP_SLOTS 64  // fingerprint accumulators (CTAs spread their atomics over them)

template <bool SEARCH>
__global__ void k_validate(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow, const int32_t *__restrict__ dst, uint32_t n,
                           uint32_t m, int full, int *__restrict__ status, unsigned long long *__restrict__ searched,
                           uint32_t *__restrict__ rev, unsigned long long *__restrict__ fp) {
  __shared__ accx_tile_rows<256> sh;
  __shared__ unsigned long long s_fp[2][8];
  uint32_t base = blockIdx.x * 256u;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<256>(off, tilerow, n, m, base, e, &sh);
  int flag = 0;
  bool chk = false;
  if (e < m) {
    const int32_t v = dst[e];
    if (v < 0 || (uint32_t)v >= n) {
      flag = V_RANGE;
    } else if (full) {
      if ((uint32_t)v == u) {
        flag = V_SELF;
      } else if (e > off[u] && dst[e - 1] >= v) {
        flag = V_UNSORTED;
      } else if (SEARCH) {
        const uint32_t du = off[u + 1] - off[u], b = off[v], t = off[v + 1], dv = t - b;
        chk = dv < du || (dv == du && (uint32_t)v > u);
        if (chk) {
          const uint32_t r = accx_lower_bound(dst, b, t, (int32_t)u);
          if (r >= t || dst[r] != (int32_t)u) {
            flag = V_ASYM;
          } else if (rev) {  // a valid graph's pairs cover every entry: the reverse index for free
            rev[e] = r;
            rev[r] = e;
          }
        }
      }
    }
  }
  if (flag) atomicOr(status, flag);
  if (SEARCH && full) {  // uniform over the block
    const int c = __syncthreads_count(chk);
    if (threadIdx.x == 0 && c) atomicAdd(searched, (unsigned long long)c);
  }
  if (fp) {  // uniform over the grid: the fingerprints of this block's entries
    unsigned long long d1 = 0, d2 = 0;
    if (e < m && !flag) {
      const unsigned long long v = (uint32_t)dst[e];
      const unsigned long long a = ((unsigned long long)u << 32) | v, b = (v << 32) | u;
      d1 = fp_splitmix(a) - fp_splitmix(b);
      d2 = fp_fmix(a) - fp_fmix(b);
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
      d1 += __shfl_xor_sync(ACCX_FULL_MASK, d1, d);
      d2 += __shfl_xor_sync(ACCX_FULL_MASK, d2, d);
    }
    if ((threadIdx.x & 31) == 0) {
      s_fp[0][threadIdx.x >> 5] = d1;
      s_fp[1][threadIdx.x >> 5] = d2;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
      unsigned long long t = 0;
      for (int w = 0; w < 8; w++) t += s_fp[threadIdx.x][w];
      if (t) atomicAdd(&fp[threadIdx.x * FP_SLOTS + blockIdx.x % FP_SLOTS], t);  // wraps mod 2^64
    }
  }
}

__global__ void k_iota(uint32_t *__restrict__ v, uint32_t m) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) v[i] = i;
}

// The reverse index by a stable radix sort of (neighbour id, entry index) pairs
// over the id bits.  The sort keeps the row order (w ascending) of the entries
// (w, v) of one neighbour v, so on a symmetric CSR with sorted rows the run of v
// is row v's place and the entry sorted to place i is the reverse of entry i:
// the sorted indices ARE the reverse index (an involution, so it is its own
// inverse).  k_rev_check verifies that premise at every place i instead of
// assuming it:
//   key[i] == row(i)                    every vertex is the neighbour in as many
//                                       entries as its own row is long;
//   off[dst[i]] <= rev[i] < off[dst[i]+1]  the entry e = rev[i] = (w, v) sorted
//                                       to place i lies in the row of place i's
//                                       neighbour: w = dst[i].
// Together entry i = (v, w) is the reverse of e, and since rev is a permutation
// of [0, m) every entry has its reverse: the graph is symmetric.  The second
// test reads off[] at neighbour ids, an array of 4(n+1) bytes that the L2 holds
// for graphs of up to ~30M vertices, where a test through rev itself would be a
// random read of the 4m-byte index.
__global__ void __launch_bounds__(256) k_rev_check(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow,
                                                   const int32_t *__restrict__ dst, uint32_t n, uint32_t m,
                                                   const uint32_t *__restrict__ key, const uint32_t *__restrict__ rev,
                                                   int *__restrict__ status) {
  __shared__ accx_tile_rows<256> sh;
  const uint32_t base = blockIdx.x * 256u;
  const uint32_t i = base + threadIdx.x;
  const uint32_t u = accx_tile_row<256>(off, tilerow, n, m, base, i, &sh);
  if (i < m) {
    const uint32_t v = (uint32_t)dst[i], r = rev[i];  // v < n: the range check ran first
    if (key[i] != u || r < __ldg(off + v) || r >= __ldg(off + v + 1)) atomicOr(status, V_ASYM);
  }
}

// The sort behind k_rev_check, for the CSR (off, tilerow, dst) of g with g->m
// entries, all ids already range-checked.  About 16 bytes per entry of scratch.
// With d_status the premise is checked (defects OR-ed into *d_status, the caller
// reads it); without it the CSR must be known symmetric.  On success *rev_out is
// a new device array (the caller owns it) -- valid as a reverse index only if
// the check passed or the CSR is symmetric.  Returns ACCX_ERR_OOM, before any
// work, when the scratch does not fit.
int accx_rev_by_sort(accx_graph *g, const uint32_t *off, const uint32_t *tilerow, const int32_t *dst, int *d_status,
                     cudaStream_t s, uint32_t **rev_out) {
  const uint32_t m = (uint32_t)g->m;
  *rev_out = nullptr;
  if (!m) return ACCX_OK;
  int bits = 1;
  while (bits < 32 && (1ull << bits) < (unsigned long long)g->n) bits++;
  uint32_t *buf[4] = {nullptr, nullptr, nullptr, nullptr};
  void *tmp = nullptr;
  size_t tb = 0;
  cub::DoubleBuffer<uint32_t> dk(nullptr, nullptr), dv(nullptr, nullptr);
  if (cub::DeviceRadixSort::SortPairs(nullptr, tb, dk, dv, (int64_t)m, 0, bits, s) != cudaSuccess) {
    accx_set_cuda_error(cudaGetLastError(), "rev sort", __FILE__, __LINE__);
    return ACCX_ERR_CUDA;
  }
  bool room = true;
  for (int i = 0; i < 4 && room; i++)
    room = accx_dev_alloc((void **)&buf[i], sizeof(uint32_t) * (size_t)m, nullptr) == cudaSuccess;
  if (room) room = accx_dev_alloc(&tmp, tb + 16, nullptr) == cudaSuccess;
  if (!room) {
    cudaGetLastError();
    for (uint32_t *p : buf) accx_dev_free(p, nullptr);
    accx_dev_free(tmp, nullptr);
    return ACCX_ERR_OOM;
  }
  int rc = ACCX_OK;
  dk = cub::DoubleBuffer<uint32_t>(buf[0], buf[1]);
  dv = cub::DoubleBuffer<uint32_t>(buf[2], buf[3]);
  if (cudaMemcpyAsync(buf[0], dst, sizeof(uint32_t) * (size_t)m, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    rc = ACCX_ERR_CUDA;
  if (!rc) {
    k_iota<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(buf[2], m);
    if (cub::DeviceRadixSort::SortPairs(tmp, tb, dk, dv, (int64_t)m, 0, bits, s) != cudaSuccess) rc = ACCX_ERR_CUDA;
  }
  if (!rc && d_status)
    k_rev_check<<<(m + 255) / 256, 256, 0, s>>>(off, tilerow, dst, g->n, m, dk.Current(), dv.Current(), d_status);
  if (!rc && (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)) rc = ACCX_ERR_CUDA;
  if (rc) {
    accx_set_cuda_error(cudaGetLastError(), "rev sort", __FILE__, __LINE__);
    cudaStreamSynchronize(s);  // nothing may still read the buffers
  }
  uint32_t *keep = rc ? nullptr : dv.Current();
  for (uint32_t *p : buf)
    if (p != keep) accx_dev_free(p, nullptr);
  accx_dev_free(tmp, nullptr);
  *rev_out = keep;
  return rc;
}

__global__ void k_tilerow(const uint32_t *__restrict__ off, uint32_t n, uint32_t m, uint32_t ntiles,
                          uint32_t *__restrict__ tr) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles; t += gridDim.x * blockDim.x) {
    uint32_t e = t < ntiles ? t * 256u : m - 1;
    if (e >= m) e = m - 1;
    tr[t] = accx_row_of(off, 0, n, e);
  }
}

int accx_tilerow_build(accx_graph *g, const uint32_t *off, uint32_t **out, cudaStream_t s) {
  const uint32_t m = (uint32_t)g->m;
  if (m == 0 || *out) return ACCX_OK;
  const uint32_t ntiles = (m + 255) / 256;
  uint32_t *p = nullptr;
  ACCX_CUDA_TRY(accx_dev_alloc((void **)&p, sizeof(uint32_t) * ((size_t)ntiles + 2), g->home));
  if (g->home && g->home != s) ACCX_CUDA_TRY(cudaStreamSynchronize(g->home));
  k_tilerow<<<accx_sm_count(g->device) * 8, 256, 0, s>>>(off, g->n, m, ntiles, p);
  ACCX_CUDA_TRY(cudaGetLastError());
  *out = p;
  return ACCX_OK;
}

__global__ void k_check_offsets(const uint32_t *__restrict__ off, uint32_t n, uint32_t m, int *status) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (off[i + 1] < off[i]) atomicOr(status, V_RANGE);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (off[0] != 0 || off[n] != m)) atomicOr(status, V_RANGE);
}

// full: the order, self-loop and symmetry checks besides the range checks;
// exact: symmetry by the sort (accx_rev_by_sort, which also records the reverse
// index) instead of the fingerprints.
int accx_graph_validate_device(accx_graph *g, int full, int exact, cudaStream_t s) {
  // [0] defect bits, [2..3] searched-entry count, then 2 x FP_SLOTS fingerprint sums
  const size_t words = 4 + 4 * FP_SLOTS;
  int *d_status = nullptr;
  ACCX_CUDA_TRY(cudaMalloc(&d_status, words * sizeof(int)));
  unsigned long long *d_searched = reinterpret_cast<unsigned long long *>(d_status + 2);
  unsigned long long *d_fp = reinterpret_cast<unsigned long long *>(d_status + 4);
  int rc = ACCX_OK;
  do {
    if (cudaMemsetAsync(d_status, 0, words * sizeof(int), s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    k_check_offsets<<<accx_grid_for(g->device, 256, 4), 256, 0, s>>>(g->d_off, g->n, (uint32_t)g->m, d_status);
    int st = 0;
    if (cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (st) { rc = ACCX_ERR_RANGE; break; }
    if ((rc = accx_tilerow_build(g, g->d_off, &g->d_tilerow, s)) != ACCX_OK) break;
    if (!g->m) {
      if (full) g->symmetric = true;
      break;
    }
    const uint32_t blocks = (uint32_t)((g->m + 255) / 256);
    const bool fingerprints = full && !exact;
    k_validate<false><<<blocks, 256, 0, s>>>(g->d_off, g->d_tilerow, g->d_dst, g->n, (uint32_t)g->m, full, d_status,
                                             nullptr, nullptr, fingerprints ? d_fp : nullptr);
    unsigned long long fp[2 * FP_SLOTS];
    if (cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        (fingerprints && cudaMemcpyAsync(fp, d_fp, sizeof(fp), cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if (fingerprints && !st) {
      unsigned long long f1 = 0, f2 = 0;
      for (int i = 0; i < FP_SLOTS; i++) {
        f1 += fp[i];
        f2 += fp[FP_SLOTS + i];
      }
      if (f1 || f2) st = V_ASYM;
    }
    if (full && exact && !st) {
      // symmetry, and with it the reverse index, by the sort; by a search per
      // entry pair when its scratch does not fit
      uint32_t *rev = nullptr;
      rc = g->d_rev_orig ? ACCX_ERR_OOM : accx_rev_by_sort(g, g->d_off, g->d_tilerow, g->d_dst, d_status, s, &rev);
      if (rc == ACCX_ERR_OOM) {
        rc = ACCX_OK;
        if (!g->d_rev_orig && accx_dev_alloc((void **)&rev, sizeof(uint32_t) * (size_t)g->m, nullptr) != cudaSuccess) {
          cudaGetLastError();
          rev = nullptr;  // no room: counts build the index themselves
        }
        k_validate<true><<<blocks, 256, 0, s>>>(g->d_off, g->d_tilerow, g->d_dst, g->n, (uint32_t)g->m, full, d_status,
                                                d_searched, rev, nullptr);
        unsigned long long searched = 0;
        if (cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(&searched, d_searched, sizeof(searched), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
          accx_dev_free(rev, nullptr);
          rc = ACCX_ERR_CUDA;
          break;
        }
        if (!st && 2 * searched != g->m) st = V_ASYM;
      } else if (rc == ACCX_OK) {
        if (cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
          accx_dev_free(rev, nullptr);
          rc = ACCX_ERR_CUDA;
          break;
        }
      } else {
        break;
      }
      if (rev) {
        if (!st) g->d_rev_orig = rev;  // complete only for a graph that passed
        else accx_dev_free(rev, nullptr);
      }
    }
    if (full && !st) g->symmetric = true;
    rc = (st & V_RANGE) ? ACCX_ERR_RANGE : (st & V_SELF) ? ACCX_ERR_SELF_LOOP
       : (st & V_UNSORTED) ? ACCX_ERR_UNSORTED : (st & V_ASYM) ? ACCX_ERR_ASYMMETRIC : ACCX_OK;
  } while (0);
  cudaFree(d_status);
  if (rc == ACCX_ERR_CUDA) accx_set_cuda_error(cudaGetLastError(), "validate", __FILE__, __LINE__);
  return rc;
}

static int alloc_graph(uint32_t n, uint64_t m, accx_graph **out) {
  if (m >= (1ull << 32) - ACCX_DST_PAD) return ACCX_ERR_TOO_LARGE;
  int dev = 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return ACCX_ERR_NO_DEVICE;
  }
  ACCX_CUDA_TRY(cudaGetDevice(&dev));
  accx_graph *g = new (std::nothrow) accx_graph();
  if (!g) return ACCX_ERR_OOM;
  g->device = dev;
  g->n = n;
  g->m = m;
  if (accx_dev_alloc((void **)&g->d_off, sizeof(uint32_t) * ((size_t)n + 1), nullptr) != cudaSuccess ||
      accx_dev_alloc((void **)&g->d_dst, sizeof(int32_t) * ((size_t)m + ACCX_DST_PAD), nullptr) != cudaSuccess) {
    cudaGetLastError();
    accx_graph_free(g);
    return ACCX_ERR_OOM;
  }
  // The padding reads as ids that match nothing.
  if (cudaMemset(g->d_dst + m, 0xff, sizeof(int32_t) * ACCX_DST_PAD) != cudaSuccess) {
    accx_graph_free(g);
    return ACCX_ERR_CUDA;
  }
  *out = g;
  return ACCX_OK;
}

extern "C" int accx_graph_create(const uint32_t *off, const int32_t *dst, uint32_t n, uint64_t m, unsigned flags,
                                 void *stream, accx_graph **out) {
  if (!off || (!dst && m) || !out) return ACCX_ERR_INVALID_ARG;
  *out = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  // the offsets are checked on the device (k_check_offsets) before any kernel
  // indexes with them
  accx_graph *g = nullptr;
  int rc = alloc_graph(n, m, &g);
  if (rc) return rc;
  rc = accx_copy_in(g->d_off, off, sizeof(uint32_t) * ((size_t)n + 1), s);
  if (!rc) rc = accx_copy_in(g->d_dst, dst, sizeof(int32_t) * (size_t)m, s);
  if (!rc) rc = accx_graph_validate_device(g, (flags & ACCX_GRAPH_VALIDATE) ? 1 : 0,
                                           (flags & ACCX_GRAPH_VALIDATE_EXACT) ? 1 : 0, s);
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { accx_set_cuda_error(e, "create", __FILE__, __LINE__); rc = ACCX_ERR_CUDA; }
  }
  if (rc) { accx_graph_free(g); return rc; }
  *out = g;
  return ACCX_OK;
}

extern "C" int accx_graph_load_dir(const char *dir, unsigned flags, void *stream, accx_graph **out) {
  if (!dir || !out) return ACCX_ERR_INVALID_ARG;
  *out = nullptr;
  std::string d(dir);
  FILE *f = fopen((d + "/b_degree.bin").c_str(), "rb");
  if (!f) return ACCX_ERR_IO;
  int32_t int_size = 0;
  uint32_t n = 0, m = 0;
  if (fread(&int_size, 4, 1, f) != 1 || fread(&n, 4, 1, f) != 1 || fread(&m, 4, 1, f) != 1) {
    fclose(f);
    return ACCX_ERR_IO;
  }
  std::vector<uint32_t> off((size_t)n + 1);
  std::vector<int32_t> deg(n);
  size_t got = n ? fread(deg.data(), 4, n, f) : 0;
  fclose(f);
  if (got != n) return ACCX_ERR_IO;
  uint64_t acc = 0;
  off[0] = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (deg[i] < 0) return ACCX_ERR_RANGE;
    acc += (uint32_t)deg[i];
    if (acc > m) return ACCX_ERR_RANGE;
    off[i + 1] = (uint32_t)acc;
  }
  if (acc != m) return ACCX_ERR_RANGE;
  f = fopen((d + "/b_adj.bin").c_str(), "rb");
  if (!f) return ACCX_ERR_IO;
  int32_t *h_dst = nullptr;
  if (cudaMallocHost(&h_dst, sizeof(int32_t) * ((size_t)m + 1)) != cudaSuccess) {
    cudaGetLastError();
    fclose(f);
    return ACCX_ERR_OOM;
  }
  got = m ? fread(h_dst, 4, m, f) : 0;
  fclose(f);
  int rc = (got == m) ? ACCX_OK : ACCX_ERR_IO;
  if (!rc) rc = accx_graph_create(off.data(), h_dst, n, m, flags, stream, out);
  cudaFreeHost(h_dst);
  return rc;
}

extern "C" int accx_graph_free(accx_graph *g) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  void *ptrs[] = {g->d_off,      g->d_dst,    g->d_cnt,  g->d_edge_list, g->d_icnt,  g->d_prefix, g->d_scan_tmp,
                  g->d_counters, g->d_table,  g->d_roff, g->d_rdst,      g->d_rmap,  g->d_rcnt,   g->d_oldid,
                  g->d_newid,    g->d_simkey, g->d_tilerow, g->d_rtilerow, g->d_src, g->d_pre, g->d_or_sl, g->d_or_items, g->d_rev, g->d_rev_orig, g->d_vinfo};
  accx_query_ctx_release(&g->qc);
  for (void *p : ptrs) accx_dev_free(p, g->home);
  for (int i = 0; i <= ACCX_NUM_PHASES; i++)
    if (g->ev[i]) cudaEventDestroy(g->ev[i]);
  accx_model_release(g);
  delete g;
  return ACCX_OK;
}

extern "C" int accx_graph_size(const accx_graph *g, uint32_t *n, uint64_t *m) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  if (n) *n = g->n;
  if (m) *m = g->m;
  return ACCX_OK;
}

extern "C" int accx_graph_download(const accx_graph *g, uint32_t *off, int32_t *dst, void *stream) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (off) {
    int rc = accx_copy_out(off, g->d_off, sizeof(uint32_t) * ((size_t)g->n + 1), s);
    if (rc) return rc;
  }
  if (dst) {
    int rc = accx_copy_out(dst, g->d_dst, sizeof(int32_t) * (size_t)g->m, s);
    if (rc) return rc;
  }
  return ACCX_OK;
}

extern "C" int accx_graph_device_ptrs(const accx_graph *g, const uint32_t **off, const int32_t **dst,
                                      const int32_t **cnt) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  if (off) *off = g->d_off;
  if (dst) *dst = g->d_dst;
  if (cnt) *cnt = g->cnt_valid ? g->d_cnt : nullptr;
  return ACCX_OK;
}

extern "C" int accx_write_graph_dir(const char *dir, const uint32_t *off, const int32_t *dst, uint32_t n,
                                    uint64_t m) {
  if (!dir || !off || (!dst && m)) return ACCX_ERR_INVALID_ARG;
  if (m >= (1ull << 32)) return ACCX_ERR_TOO_LARGE;
  std::string d(dir);
  FILE *f = fopen((d + "/b_degree.bin").c_str(), "wb");
  if (!f) return ACCX_ERR_IO;
  int32_t int_size = 4;
  uint32_t n32 = n, m32 = (uint32_t)m;
  bool ok = fwrite(&int_size, 4, 1, f) == 1 && fwrite(&n32, 4, 1, f) == 1 && fwrite(&m32, 4, 1, f) == 1;
  std::vector<int32_t> deg(n);
  for (uint32_t i = 0; i < n; i++) deg[i] = (int32_t)(off[i + 1] - off[i]);
  if (n) ok = ok && fwrite(deg.data(), 4, n, f) == n;
  ok = (fclose(f) == 0) && ok;
  if (!ok) return ACCX_ERR_IO;
  f = fopen((d + "/b_adj.bin").c_str(), "wb");
  if (!f) return ACCX_ERR_IO;
  ok = m ? fwrite(dst, 4, m, f) == m : true;
  ok = (fclose(f) == 0) && ok;
  return ok ? ACCX_OK : ACCX_ERR_IO;
}

// All-edge common-neighbour counting that allocates no memory.
//
// Some callers cannot call cudaMalloc: code running inside a stream-ordered
// memory pool budget set by a host framework, plugins loaded into a process
// whose allocator owns all device memory (and fails or deadlocks on a foreign
// cudaMalloc), or real-time loops that must not hit the driver's allocator.
// accx_cn_count_noalloc serves them: the caller passes the device CSR and the
// device output array, and the only scratch the computation needs -- the list of
// owned edges and its length counter -- lives in the file-scope array below,
// which every GPU that loads this library holds until the process exits.
//
// The computation is the merge variant of accx_cn_count: a classify pass
// appends each owned edge (the endpoint with the larger degree, ties: smaller
// id) to the scratch list, and one warp per listed edge counts the intersection
// with the shared merge-path routine and writes the value (plus bias) to both
// the entry and its reverse entry.
#include <mutex>

#include "accx_internal.h"
#include "devutil.cuh"
#include "merge.cuh"

// Owned edges the scratch list can hold; a symmetric graph has m/2 owned edges,
// so graphs up to 2 * ACCX_NOALLOC_MAX_OWNED CSR entries fit.
#define ACCX_NOALLOC_MAX_OWNED (1u << 20)

// [0, MAX): owned edges as (u, e); [MAX].x: the list length (an append
// counter), [MAX].y: set to 1 when owned edges did not fit the list.  That can
// only happen on an asymmetric CSR, which this entry point does not check: a
// symmetric one has exactly m/2 owned edges.  8 MiB + 8 bytes per device.
static __device__ __align__(256) uint2 g_noalloc_scratch[ACCX_NOALLOC_MAX_OWNED + 1];

template <int TILE>
__global__ void __launch_bounds__(TILE) k_noalloc_classify(const uint32_t *__restrict__ off,
                                                           const int32_t *__restrict__ dst, uint32_t n, uint32_t m,
                                                           uint2 *__restrict__ scratch) {
  __shared__ accx_tile_rows<TILE> sh;
  uint32_t base = blockIdx.x * (uint32_t)TILE;
  uint32_t e = base + threadIdx.x;
  uint32_t u = accx_tile_row<TILE>(off, nullptr, n, m, base, e, &sh);
  bool own = false;
  if (e < m) {
    uint32_t v = (uint32_t)dst[e];
    own = accx_owns(u, off[u + 1] - off[u], v, off[v + 1] - off[v]);
  }
  const unsigned mask = __ballot_sync(ACCX_FULL_MASK, own);
  if (!mask) return;
  const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
  uint32_t p = 0;
  if (lane == leader) p = atomicAdd(&scratch[ACCX_NOALLOC_MAX_OWNED].x, (uint32_t)__popc(mask));
  p = __shfl_sync(ACCX_FULL_MASK, p, leader);
  if (own) {
    uint32_t idx = p + __popc(mask & ((1u << lane) - 1u));
    if (idx < ACCX_NOALLOC_MAX_OWNED) scratch[idx] = make_uint2(u, e);
    else scratch[ACCX_NOALLOC_MAX_OWNED].y = 1u;  // dropped: asymmetric input
  }
}

__global__ void __launch_bounds__(256) k_noalloc_merge(const uint32_t *__restrict__ off,
                                                        const int32_t *__restrict__ dst,
                                                        const uint2 *__restrict__ scratch, int32_t bias,
                                                        int32_t *__restrict__ cnt) {
  __shared__ __align__(16) int32_t buf[8][2][MERGE_WIN];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t total = scratch[ACCX_NOALLOC_MAX_OWNED].x;
  if (total > ACCX_NOALLOC_MAX_OWNED) total = ACCX_NOALLOC_MAX_OWNED;
  const uint32_t nw = gridDim.x * 8u;
  for (uint32_t it = blockIdx.x * 8u + (uint32_t)w; it < total; it += nw) {
    const uint2 p = scratch[it];
    const uint32_t u = p.x, e = p.y, v = (uint32_t)dst[e];
    const uint32_t vb = off[v], ve = off[v + 1];
    const uint32_t c = accx_warp_merge_count(dst, off[u], off[u + 1], vb, ve, buf[w][0], buf[w][1], lane);
    if (lane == 0) {
      const int32_t val = (int32_t)c + bias;
      cnt[e] = val;
      const uint32_t r = accx_lower_bound(dst, vb, ve, (int32_t)u);
      if (r < ve && dst[r] == (int32_t)u) cnt[r] = val;
    }
    __syncwarp();
  }
}

// Device address of the scratch array, looked up once per device (with that
// device current) and cached.
static std::mutex g_noalloc_mu;
static uint2 *g_noalloc_ptr[64];

static int noalloc_scratch(int dev, uint2 **out) {
  if (dev < 0 || dev >= 64) return ACCX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      accx_set_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
      return ACCX_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = static_cast<uint2 *>(p);
  }
  *out = g_noalloc_ptr[dev];
  return ACCX_OK;
}

extern "C" uint64_t accx_cn_count_noalloc_max_entries(void) { return 2ull * ACCX_NOALLOC_MAX_OWNED; }

extern "C" int accx_cn_count_noalloc(const uint32_t *off, const int32_t *dst, uint32_t n, uint64_t m, int32_t bias,
                                     int32_t *cnt, void *stream) {
  if (!off || (m && (!dst || !cnt))) return ACCX_ERR_INVALID_ARG;
  if (m > 2ull * ACCX_NOALLOC_MAX_OWNED) return ACCX_ERR_TOO_LARGE;
  if (!accx_is_device_ptr(off) || (m && (!accx_is_device_ptr(dst) || !accx_is_device_ptr(cnt))))
    return ACCX_ERR_INVALID_ARG;  // staging host arrays would need an allocation
  int dev = 0;
  ACCX_CUDA_TRY(cudaGetDevice(&dev));
  uint2 *scratch = nullptr;
  int rc = noalloc_scratch(dev, &scratch);
  if (rc) return rc;
  if (m == 0 || n == 0) return ACCX_OK;
  cudaStream_t s = (cudaStream_t)stream;
  // the list length and the overflow flag start at zero on every call (the array
  // keeps the last call's contents)
  ACCX_CUDA_TRY(cudaMemsetAsync(scratch + ACCX_NOALLOC_MAX_OWNED, 0, sizeof(uint2), s));
  const uint32_t m32 = (uint32_t)m;
  k_noalloc_classify<256><<<(m32 + 255) / 256, 256, 0, s>>>(off, dst, n, m32, scratch);
  k_noalloc_merge<<<accx_sm_count(dev) * 8, 256, 0, s>>>(off, dst, scratch, bias, cnt);
  ACCX_CUDA_TRY(cudaGetLastError());
  return ACCX_OK;
}

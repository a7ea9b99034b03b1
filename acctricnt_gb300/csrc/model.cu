// Learned kernel scheduler: a small MLP cost model per degree bucket.
//
// Network: ACCX_MODEL_IN features -> 32 ReLU -> 32 ReLU -> one output per
// kernel kind (predicted log2 seconds per edge).  Parameters live on the device
// as an FP32 master copy (updated by Adam) and the FP16 weights every forward
// pass reads; all products accumulate in FP32.  The kernels here are the
// library's own:
//   k_model_grad     forward + backward of a batch (one thread per sample),
//                    gradient summed in shared memory, then globally;
//   k_model_adam     the optimizer step, refreshing the FP16 copy;
//   k_model_infer    register-resident inference: a warp keeps one hidden unit's
//                    weights per lane in registers for the whole launch and
//                    evaluates rows with shuffles; with a graph's bucket features
//                    it writes the argmin kind of every bucket straight into the
//                    handle's kernel table, so ACCX_POLICY_MODEL needs no host
//                    round trip.
#include <cuda_fp16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "accx_internal.h"
#include "devutil.cuh"

#define IN ACCX_MODEL_IN
#define H ACCX_MODEL_H
#define OUT ACCX_MODEL_OUT
#define NP ACCX_MODEL_NPARAMS
#define O_W1 0
#define O_B1 (IN * H)
#define O_W2 (O_B1 + H)
#define O_B2 (O_W2 + H * H)
#define O_W3 (O_B2 + H)
#define O_B3 (O_W3 + H * OUT)

static_assert(O_B3 + OUT == NP, "parameter layout");

struct accx_model {
  int device = 0;
  float *d_master = nullptr;  // NP fp32
  __half *d_w = nullptr;      // NP fp16 (what the forward pass reads)
  float *d_m = nullptr, *d_v = nullptr;  // Adam moments
  float *d_grad = nullptr;    // NP
  float *d_loss = nullptr;    // 1
  int step = 0;
  float bias[OUT] = {0.f, 0.f, 0.f};  // per-kind log2 offsets added before the argmin of a table
};

struct accx_kind_bias {
  float b[OUT];
};

// ---------------------------------------------------------------------------
__global__ void k_to_half(const float *__restrict__ src, __half *__restrict__ dst, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = __float2half_rn(src[i]);
}

// Forward + backward of the mean squared error on the output of each sample's
// kind.  grad and loss are accumulated (the caller zeroes them).
__global__ void __launch_bounds__(128) k_model_grad(const __half *__restrict__ w, const float *__restrict__ x,
                                                    const int32_t *__restrict__ kind, const float *__restrict__ target,
                                                    uint32_t k, float *__restrict__ grad, float *__restrict__ loss) {
  __shared__ float sw[NP];
  __shared__ float sg[NP];
  __shared__ float sl;
  for (int i = threadIdx.x; i < NP; i += blockDim.x) {
    sw[i] = __half2float(w[i]);
    sg[i] = 0.f;
  }
  if (threadIdx.x == 0) sl = 0.f;
  __syncthreads();
  const float inv = 1.f / (float)k;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < k; s += gridDim.x * blockDim.x) {
    float xi[IN], h1[H], h2[H];
#pragma unroll
    for (int f = 0; f < IN; f++) xi[f] = x[(size_t)s * IN + f];
#pragma unroll
    for (int j = 0; j < H; j++) {
      float a = sw[O_B1 + j];
#pragma unroll
      for (int f = 0; f < IN; f++) a = fmaf(xi[f], sw[O_W1 + f * H + j], a);
      h1[j] = a > 0.f ? a : 0.f;
    }
#pragma unroll
    for (int j = 0; j < H; j++) {
      float a = sw[O_B2 + j];
#pragma unroll
      for (int i = 0; i < H; i++) a = fmaf(h1[i], sw[O_W2 + i * H + j], a);
      h2[j] = a > 0.f ? a : 0.f;
    }
    const int o = kind[s];
    float y = sw[O_B3 + o];
#pragma unroll
    for (int j = 0; j < H; j++) y = fmaf(h2[j], sw[O_W3 + j * OUT + o], y);
    const float err = y - target[s];
    atomicAdd(&sl, err * err * inv);
    const float dy = 2.f * err * inv;
    atomicAdd(&sg[O_B3 + o], dy);
    float dh2[H];
#pragma unroll
    for (int j = 0; j < H; j++) {
      atomicAdd(&sg[O_W3 + j * OUT + o], h2[j] * dy);
      dh2[j] = h2[j] > 0.f ? sw[O_W3 + j * OUT + o] * dy : 0.f;
      atomicAdd(&sg[O_B2 + j], dh2[j]);
    }
#pragma unroll
    for (int i = 0; i < H; i++) {
      float d1 = 0.f;
#pragma unroll
      for (int j = 0; j < H; j++) {
        atomicAdd(&sg[O_W2 + i * H + j], h1[i] * dh2[j]);
        d1 = fmaf(sw[O_W2 + i * H + j], dh2[j], d1);
      }
      d1 = h1[i] > 0.f ? d1 : 0.f;
      atomicAdd(&sg[O_B1 + i], d1);
#pragma unroll
      for (int f = 0; f < IN; f++) atomicAdd(&sg[O_W1 + f * H + i], xi[f] * d1);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NP; i += blockDim.x)
    if (sg[i] != 0.f) atomicAdd(&grad[i], sg[i]);
  if (threadIdx.x == 0) atomicAdd(loss, sl);
}

__global__ void k_model_adam(float *__restrict__ master, __half *__restrict__ w, float *__restrict__ mm,
                             float *__restrict__ vv, const float *__restrict__ grad, float lr, float b1t, float b2t) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x) {
    float g = grad[i];
    float m = b1 * mm[i] + (1.f - b1) * g;
    float v = b2 * vv[i] + (1.f - b2) * g * g;
    mm[i] = m;
    vv[i] = v;
    float mh = m / (1.f - b1t), vh = v / (1.f - b2t);
    float p = master[i] - lr * mh / (sqrtf(vh) + eps);
    master[i] = p;
    w[i] = __float2half_rn(p);
  }
}

// Register-resident inference.  Lane j of every warp holds hidden unit j's
// weights (W1[:,j], b1[j], W2[:,j], b2[j], W3[j,:]) in registers for the whole
// launch; a row's first layer is per lane, the second gathers the 32 first-layer
// activations by shuffles, the output layer is a warp sum.  With `table` set the
// rows are a graph's bucket features and the argmin kind of every populated
// bucket is written to table[row] (and, with `cost` set, the bucket's predicted
// time in seconds, edges x 2^(the chosen kind's output), to cost[row]); otherwise
// the outputs go to y.
__global__ void __launch_bounds__(256) k_model_infer(const __half *__restrict__ w, const float *__restrict__ x,
                                                     uint32_t k, float *__restrict__ y,
                                                     const unsigned long long *__restrict__ edges,
                                                     uint8_t *__restrict__ table, accx_kind_bias kb,
                                                     double *__restrict__ cost = nullptr) {
  const int lane = threadIdx.x & 31;
  float w1[IN], w2[H], w3[OUT], b3[OUT];
#pragma unroll
  for (int f = 0; f < IN; f++) w1[f] = __half2float(w[O_W1 + f * H + lane]);
  const float b1 = __half2float(w[O_B1 + lane]);
#pragma unroll
  for (int i = 0; i < H; i++) w2[i] = __half2float(w[O_W2 + i * H + lane]);
  const float b2 = __half2float(w[O_B2 + lane]);
#pragma unroll
  for (int o = 0; o < OUT; o++) {
    w3[o] = __half2float(w[O_W3 + lane * OUT + o]);
    b3[o] = __half2float(w[O_B3 + o]);
  }
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < k; r += warps) {
    float a = b1;
#pragma unroll
    for (int f = 0; f < IN; f++) a = fmaf(x[(size_t)r * IN + f], w1[f], a);
    const float h1 = a > 0.f ? a : 0.f;
    float a2 = b2;
#pragma unroll
    for (int i = 0; i < H; i++) a2 = fmaf(__shfl_sync(ACCX_FULL_MASK, h1, i), w2[i], a2);
    const float h2 = a2 > 0.f ? a2 : 0.f;
    float out[OUT];
#pragma unroll
    for (int o = 0; o < OUT; o++) {
      float p = h2 * w3[o];
#pragma unroll
      for (int d = 16; d >= 1; d >>= 1) p += __shfl_xor_sync(ACCX_FULL_MASK, p, d);
      out[o] = p + b3[o];
    }
    if (lane == 0) {
      if (table) {
        int best = 0;
#pragma unroll
        for (int o = 1; o < OUT; o++)
          if (out[o] + kb.b[o] < out[best] + kb.b[best]) best = o;
        table[r] = (edges && edges[r] == 0) ? (uint8_t)ACCX_KIND_MERGE : (uint8_t)best;
        if (cost) cost[r] = (edges && edges[r]) ? (double)edges[r] * exp2((double)out[best]) : 0.0;
      } else {
#pragma unroll
        for (int o = 0; o < OUT; o++) y[(size_t)r * OUT + o] = out[o];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Bucket statistics over owned edges, both modes in one pass over the CSR counts
// run on: [0] direct (owners and buckets by degree), [1] oriented (by prefix
// length pre[], edges whose smaller prefix is empty left out -- the edges and
// sizes oriented counting works on).  Direct statistics do not depend on the
// vertex numbering: the owner is the endpoint of larger degree, and on a tie the
// bucket and both sizes are the same whichever endpoint owns, so the relabeled
// CSR gives the original CSR's figures.
#define NBB (ACCX_NB * ACCX_NB)
#define BS_EPT 8  // consecutive entries per thread

// A thread's current run of one bucket, added to the CTA's histograms (count,
// owner sizes, other sizes) when the bucket changes.  Runs are long: within a
// row the partners come in id order, which after the relabel is degree order.
struct bs_run {
  int b = -1;
  uint32_t c = 0;
  unsigned long long so = 0, sp = 0;
  __device__ __forceinline__ void flush(unsigned long long *h) {
    if (c) {
      atomicAdd(&h[b], (unsigned long long)c);
      atomicAdd(&h[NBB + b], so);
      atomicAdd(&h[2 * NBB + b], sp);
    }
    c = 0;
    so = sp = 0;
  }
  // The chunk's last run: lanes holding the same bucket add up first (a warp's
  // lanes mostly end in a few buckets, and same-address shared atomics from one
  // warp serialise).  Sizes are summed as 16-bit halves, so 32 lanes of at most
  // BS_EPT sizes each cannot overflow 32 bits.
  __device__ __forceinline__ void flush_warp(unsigned long long *h) {
    const unsigned act = __activemask();
    const int key = c ? b : -1;
    const unsigned peers = __match_any_sync(act, key);
    if (key >= 0) {
      const unsigned long long n = __reduce_add_sync(peers, c);
      const unsigned long long o = ((unsigned long long)__reduce_add_sync(peers, (unsigned)(so >> 16)) << 16) +
                                   __reduce_add_sync(peers, (unsigned)(so & 0xffffu));
      const unsigned long long q = ((unsigned long long)__reduce_add_sync(peers, (unsigned)(sp >> 16)) << 16) +
                                   __reduce_add_sync(peers, (unsigned)(sp & 0xffffu));
      if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
        atomicAdd(&h[b], n);
        atomicAdd(&h[NBB + b], o);
        atomicAdd(&h[2 * NBB + b], q);
      }
    }
    c = 0;
    so = sp = 0;
  }
  __device__ __forceinline__ void add(unsigned long long *h, int nb, uint32_t o, uint32_t p) {
    if (nb != b) {
      flush(h);
      b = nb;
    }
    c++;
    so += o;
    sp += p;
  }
};

// Threads take chunks of BS_EPT consecutive entries (grid-stride); a chunk lies
// in one 256-entry tile, whose first and last rows tilerow[] holds, so a thread
// finds its row without the CTA (no barrier per tile).  The CTA's histograms
// reach the device counters once.
template <int NT>
__global__ void __launch_bounds__(NT, 5) k_bucket_stats(const uint32_t *__restrict__ off, const uint32_t *__restrict__ tilerow,
                                                        const int32_t *__restrict__ dst, uint32_t n, uint32_t m,
                                                        const uint32_t *__restrict__ pre,
                                                        unsigned long long *__restrict__ st_direct,
                                                        unsigned long long *__restrict__ st_orient) {
  static_assert(256 % BS_EPT == 0, "chunks inside tile-row tiles");
  __shared__ unsigned long long hs[2][3 * NBB];
  for (int i = threadIdx.x; i < 6 * NBB; i += NT) (&hs[0][0])[i] = 0;
  __syncthreads();
  const uint32_t nchunks = (uint32_t)(((unsigned long long)m + BS_EPT - 1) / BS_EPT);
  for (uint32_t ch = blockIdx.x * NT + threadIdx.x; ch < nchunks; ch += gridDim.x * NT) {
    const uint32_t e0 = ch * BS_EPT;
    const uint32_t e1 = e0 + BS_EPT < m ? e0 + BS_EPT : m;
    // the partners' sizes first (independent loads in flight), then the rows
    uint32_t vv[BS_EPT], dd[BS_EPT], pp[BS_EPT];
#pragma unroll
    for (int j = 0; j < BS_EPT; j++) vv[j] = e0 + j < e1 ? (uint32_t)__ldg(dst + e0 + j) : 0u;
#pragma unroll
    for (int j = 0; j < BS_EPT; j++) {
      dd[j] = __ldg(off + vv[j] + 1) - __ldg(off + vv[j]);
      pp[j] = __ldg(pre + vv[j]);
    }
    // tilerow[k] = the row of entry 256k, its last element the row of entry m-1
    const uint32_t t = e0 / 256u;
    uint32_t u = accx_row_of(off, __ldg(tilerow + t), __ldg(tilerow + t + 1) + 1, e0);
    uint32_t rb = __ldg(off + u), re = __ldg(off + u + 1), pu = __ldg(pre + u);
    bs_run rd, ro;
#pragma unroll
    for (int j = 0; j < BS_EPT; j++) {
      const uint32_t e = e0 + j;
      if (e >= e1) break;
      while (re <= e) {  // the next non-empty row
        u++;
        rb = re;
        re = __ldg(off + u + 1);
        pu = __ldg(pre + u);
      }
      const uint32_t v = vv[j], du = re - rb, dv = dd[j], pv = pp[j];
      if (accx_owns(u, du, v, dv)) rd.add(hs[0], accx_bucket(du) * ACCX_NB + accx_bucket(dv), du, dv);
      if (pv > 0 && accx_owns(u, pu, v, pv)) ro.add(hs[1], accx_bucket(pu) * ACCX_NB + accx_bucket(pv), pu, pv);
    }
    rd.flush_warp(hs[0]);
    ro.flush_warp(hs[1]);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * NBB; i += NT) {
    if (hs[0][i]) atomicAdd(&st_direct[i], hs[0][i]);
    if (hs[1][i]) atomicAdd(&st_orient[i], hs[1][i]);
  }
}

__device__ __forceinline__ void accx_feature_row(const unsigned long long *st, int b, uint32_t n, uint64_t m,
                                                 float *x) {
  const double E = (double)st[b];
  for (int f = 0; f < IN; f++) x[f] = 0.f;
  if (E <= 0) return;
  const double mo = (double)st[NBB + b] / E, mp = (double)st[2 * NBB + b] / E;
  const double lo = log2(mo), lp = log2(mp);
  x[0] = (float)(lo / 16.0);
  x[1] = (float)(lp / 16.0);
  x[2] = (float)((lo - lp) / 16.0);
  x[3] = (float)(log2(E + 1.0) / 32.0);
  x[4] = (float)(log2((double)n + 1.0) / 32.0);
  x[5] = (float)(log2((double)m + 1.0) / 32.0);
  x[6] = (float)(lo * lp / 256.0);
  x[7] = (float)(log2(E * mp + 1.0) / 40.0);
}

__global__ void k_features(const unsigned long long *__restrict__ st, uint32_t n, uint64_t m, float *__restrict__ x) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < NBB; b += gridDim.x * blockDim.x)
    accx_feature_row(st, b, n, m, x + (size_t)b * IN);
}

// Per-handle cache: bucket statistics and features of the graph (it never
// changes), plus the attached model.
struct accx_graph_model_state {
  // [0] direct: degrees on the handle's CSR; [1] oriented: prefix lengths on the
  // CSR counts run on (recomputed when that changes, i.e. after a relabel)
  unsigned long long *d_stats[2] = {nullptr, nullptr};  // 3 * NBB each
  float *d_feat[2] = {nullptr, nullptr};                // NBB * IN each
  bool ready[2] = {false, false};
  const uint32_t *csr[2] = {nullptr, nullptr};
  accx_model *model[2] = {nullptr, nullptr};
  // plan costs (accx_model_plan_ms): a scratch table, per-bucket costs and their sum
  uint8_t *d_ptable = nullptr;
  double *d_cost = nullptr;  // NBB + 1
};

static accx_graph_model_state *state_of(accx_graph *g) {
  if (!g->model) g->model = new (std::nothrow) accx_graph_model_state();
  return static_cast<accx_graph_model_state *>(g->model);
}

void accx_model_release(accx_graph *g) {
  auto *st = static_cast<accx_graph_model_state *>(g->model);
  if (st) {
    for (int i = 0; i < 2; i++) {
      if (st->d_stats[i]) cudaFree(st->d_stats[i]);
      if (st->d_feat[i]) cudaFree(st->d_feat[i]);
    }
    if (st->d_ptable) cudaFree(st->d_ptable);
    if (st->d_cost) cudaFree(st->d_cost);
    delete st;
  }
  g->model = nullptr;
}

// Both modes' statistics and features at once, on the CSR counts run on (the
// relabeled one when the handle has it); recomputed when that changes.
static int ensure_features(accx_graph *g, cudaStream_t s, int mode) {
  accx_graph_model_state *st = state_of(g);
  if (!st) return ACCX_ERR_OOM;
  const bool rel = g->d_roff != nullptr;
  const uint32_t *off = rel ? g->d_roff : g->d_off;
  if (st->ready[mode] && st->csr[mode] == off) return ACCX_OK;
  for (int k = 0; k < 2; k++) {
    if (!st->d_stats[k]) ACCX_CUDA_TRY(cudaMalloc(&st->d_stats[k], sizeof(unsigned long long) * 3 * NBB));
    if (!st->d_feat[k]) ACCX_CUDA_TRY(cudaMalloc(&st->d_feat[k], sizeof(float) * NBB * IN));
    ACCX_CUDA_TRY(cudaMemsetAsync(st->d_stats[k], 0, sizeof(unsigned long long) * 3 * NBB, s));
  }
  const uint32_t m = (uint32_t)g->m;
  if (m) {
    int rc = accx_prefix_lengths(g, s);
    if (rc) return rc;
    const uint32_t *tilerow = rel ? g->d_rtilerow : g->d_tilerow;
    if (!tilerow) {
      rc = accx_tilerow_build(g, off, rel ? &g->d_rtilerow : &g->d_tilerow, s);
      if (rc) return rc;
      tilerow = rel ? g->d_rtilerow : g->d_tilerow;
    }
    const uint32_t tiles = (uint32_t)(((unsigned long long)m + 256 * BS_EPT - 1) / (256 * BS_EPT));
    const uint32_t grid = std::min(tiles, (uint32_t)accx_sm_count(g->device) * 5);
    k_bucket_stats<256><<<grid, 256, 0, s>>>(off, tilerow, rel ? g->d_rdst : g->d_dst, g->n, m, g->d_pre,
                                             st->d_stats[0], st->d_stats[1]);
  }
  for (int k = 0; k < 2; k++) {
    k_features<<<(NBB + 127) / 128, 128, 0, s>>>(st->d_stats[k], g->n, g->m, st->d_feat[k]);
    st->ready[k] = true;
    st->csr[k] = off;
  }
  ACCX_CUDA_TRY(cudaGetLastError());
  return ACCX_OK;
}

// The handle's ACCX_POLICY_MODEL table, computed on the device into g->d_table.
int accx_model_table_device(accx_graph *g, cudaStream_t s, int orient) {
  accx_graph_model_state *st = state_of(g);
  const int mode = orient ? 1 : 0;
  if (!st || !st->model[mode]) return ACCX_ERR_NOT_READY;
  int rc = ensure_features(g, s, mode);
  if (rc) return rc;
  accx_kind_bias kb;
  for (int o = 0; o < OUT; o++) kb.b[o] = st->model[mode]->bias[o];
  k_model_infer<<<8, 256, 0, s>>>(st->model[mode]->d_w, st->d_feat[mode], NBB, nullptr, st->d_stats[mode], g->d_table,
                                  kb);
  ACCX_CUDA_TRY(cudaGetLastError());
  return ACCX_OK;
}

// One block sums the per-bucket costs in a fixed order (the same total on every run).
__global__ void __launch_bounds__(256) k_sum_cost(const double *__restrict__ cost, int k, double *__restrict__ out) {
  __shared__ double part[256];
  double a = 0;
  for (int i = threadIdx.x; i < k; i += 256) a += cost[i];
  part[threadIdx.x] = a;
  __syncthreads();
  for (int d = 128; d >= 1; d >>= 1) {
    if ((int)threadIdx.x < d) part[threadIdx.x] += part[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

// Predicted time (ms) of model m's own per-bucket table on g's buckets of the
// given mode: the sum over populated buckets of edges x 2^(the chosen kind's
// prediction).  The buffers live with the graph; one 8-byte copy comes back.
int accx_model_plan_ms(accx_model *m, accx_graph *g, int mode, cudaStream_t s, double *ms) {
  if (!m || !g || !ms || (mode != 0 && mode != 1)) return ACCX_ERR_INVALID_ARG;
  accx_graph_model_state *st = state_of(g);
  if (!st) return ACCX_ERR_OOM;
  int rc = ensure_features(g, s, mode);
  if (rc) return rc;
  if (!st->d_ptable) ACCX_CUDA_TRY(cudaMalloc(&st->d_ptable, NBB));
  if (!st->d_cost) ACCX_CUDA_TRY(cudaMalloc(&st->d_cost, sizeof(double) * (NBB + 1)));
  accx_kind_bias kb;
  for (int o = 0; o < OUT; o++) kb.b[o] = m->bias[o];
  k_model_infer<<<8, 256, 0, s>>>(m->d_w, st->d_feat[mode], NBB, nullptr, st->d_stats[mode], st->d_ptable, kb,
                                  st->d_cost);
  k_sum_cost<<<1, 256, 0, s>>>(st->d_cost, NBB, st->d_cost + NBB);
  double sec = 0;
  ACCX_CUDA_TRY(cudaMemcpyAsync(&sec, st->d_cost + NBB, sizeof(double), cudaMemcpyDeviceToHost, s));
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  *ms = sec * 1e3;
  return ACCX_OK;
}

int accx_model_table(accx_graph *g, uint8_t *table) {
  (void)g;
  (void)table;
  return ACCX_ERR_NOT_READY;
}

// ---------------------------------------------------------------------------
extern "C" int accx_model_create(uint64_t seed, accx_model **out) {
  if (!out) return ACCX_ERR_INVALID_ARG;
  *out = nullptr;
  accx_model *m = new (std::nothrow) accx_model();
  if (!m) return ACCX_ERR_OOM;
  cudaGetDevice(&m->device);
  if (cudaMalloc(&m->d_master, sizeof(float) * NP) != cudaSuccess || cudaMalloc(&m->d_w, sizeof(__half) * NP) != cudaSuccess ||
      cudaMalloc(&m->d_m, sizeof(float) * NP) != cudaSuccess || cudaMalloc(&m->d_v, sizeof(float) * NP) != cudaSuccess ||
      cudaMalloc(&m->d_grad, sizeof(float) * NP) != cudaSuccess || cudaMalloc(&m->d_loss, sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    accx_model_free(m);
    return ACCX_ERR_OOM;
  }
  // He-style initialisation from a counter-based stream; output bias starts at
  // -27 (about 7 ns per edge) so early predictions are in range.
  std::vector<float> p(NP, 0.f);
  uint64_t sm = seed * 0x9E3779B97F4A7C15ull + 12345;
  auto unif = [&]() {
    sm += 0x9E3779B97F4A7C15ull;
    uint64_t z = sm;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  for (int i = 0; i < IN * H; i++) p[O_W1 + i] = (float)(unif() * sqrt(6.0 / IN));
  for (int i = 0; i < H * H; i++) p[O_W2 + i] = (float)(unif() * sqrt(6.0 / H));
  for (int i = 0; i < H * OUT; i++) p[O_W3 + i] = (float)(unif() * sqrt(6.0 / H) * 0.1);
  for (int o = 0; o < OUT; o++) p[O_B3 + o] = -27.f;
  int rc = accx_model_set_params(m, p.data());
  if (rc) {
    accx_model_free(m);
    return rc;
  }
  *out = m;
  return ACCX_OK;
}

extern "C" int accx_model_free(accx_model *m) {
  if (!m) return ACCX_ERR_INVALID_ARG;
  for (void *p : {(void *)m->d_master, (void *)m->d_w, (void *)m->d_m, (void *)m->d_v, (void *)m->d_grad,
                  (void *)m->d_loss})
    if (p) cudaFree(p);
  delete m;
  return ACCX_OK;
}

extern "C" int accx_model_set_params(accx_model *m, const float *params) {
  if (!m || !params) return ACCX_ERR_INVALID_ARG;
  ACCX_CUDA_TRY(cudaMemcpy(m->d_master, params, sizeof(float) * NP, cudaMemcpyHostToDevice));
  k_to_half<<<4, 256>>>(m->d_master, m->d_w, NP);
  ACCX_CUDA_TRY(cudaMemset(m->d_m, 0, sizeof(float) * NP));
  ACCX_CUDA_TRY(cudaMemset(m->d_v, 0, sizeof(float) * NP));
  ACCX_CUDA_TRY(cudaDeviceSynchronize());
  m->step = 0;
  return ACCX_OK;
}

extern "C" int accx_model_get_params(const accx_model *m, float *params) {
  if (!m || !params) return ACCX_ERR_INVALID_ARG;
  std::vector<__half> h(NP);
  ACCX_CUDA_TRY(cudaMemcpy(h.data(), m->d_w, sizeof(__half) * NP, cudaMemcpyDeviceToHost));
  for (int i = 0; i < NP; i++) params[i] = __half2float(h[i]);
  return ACCX_OK;
}

struct dev_samples {
  float *x = nullptr, *t = nullptr;
  int32_t *k = nullptr;
  ~dev_samples() {
    if (x) cudaFree(x);
    if (t) cudaFree(t);
    if (k) cudaFree(k);
  }
};

static int upload_samples(dev_samples &d, const float *x, const int32_t *kind, const float *target, uint32_t k) {
  for (uint32_t i = 0; i < k; i++)
    if (kind[i] < 0 || kind[i] >= OUT) return ACCX_ERR_INVALID_ARG;
  ACCX_CUDA_TRY(cudaMalloc(&d.x, sizeof(float) * (size_t)k * IN));
  ACCX_CUDA_TRY(cudaMalloc(&d.t, sizeof(float) * k));
  ACCX_CUDA_TRY(cudaMalloc(&d.k, sizeof(int32_t) * k));
  ACCX_CUDA_TRY(cudaMemcpy(d.x, x, sizeof(float) * (size_t)k * IN, cudaMemcpyHostToDevice));
  ACCX_CUDA_TRY(cudaMemcpy(d.t, target, sizeof(float) * k, cudaMemcpyHostToDevice));
  ACCX_CUDA_TRY(cudaMemcpy(d.k, kind, sizeof(int32_t) * k, cudaMemcpyHostToDevice));
  return ACCX_OK;
}

static int grad_pass(accx_model *m, const dev_samples &d, uint32_t k) {
  ACCX_CUDA_TRY(cudaMemsetAsync(m->d_grad, 0, sizeof(float) * NP));
  ACCX_CUDA_TRY(cudaMemsetAsync(m->d_loss, 0, sizeof(float)));
  int blocks = (int)((k + 127) / 128);
  if (blocks > 64) blocks = 64;
  k_model_grad<<<blocks, 128>>>(m->d_w, d.x, d.k, d.t, k, m->d_grad, m->d_loss);
  ACCX_CUDA_TRY(cudaGetLastError());
  return ACCX_OK;
}

extern "C" int accx_model_loss_grad(accx_model *m, const float *x, const int32_t *kind, const float *target,
                                    uint32_t k, float *grad, float *loss) {
  if (!m || !x || !kind || !target || !k) return ACCX_ERR_INVALID_ARG;
  dev_samples d;
  int rc = upload_samples(d, x, kind, target, k);
  if (!rc) rc = grad_pass(m, d, k);
  if (rc) return rc;
  if (grad) ACCX_CUDA_TRY(cudaMemcpy(grad, m->d_grad, sizeof(float) * NP, cudaMemcpyDeviceToHost));
  if (loss) ACCX_CUDA_TRY(cudaMemcpy(loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost));
  return ACCX_OK;
}

extern "C" int accx_model_train(accx_model *m, const float *x, const int32_t *kind, const float *target, uint32_t k,
                                int epochs, float lr, float *final_loss) {
  if (!m || !x || !kind || !target || !k || epochs < 1 || !(lr > 0)) return ACCX_ERR_INVALID_ARG;
  dev_samples d;
  int rc = upload_samples(d, x, kind, target, k);
  if (rc) return rc;
  for (int ep = 0; ep < epochs; ep++) {
    rc = grad_pass(m, d, k);
    if (rc) return rc;
    m->step++;
    const float b1t = powf(0.9f, (float)m->step), b2t = powf(0.999f, (float)m->step);
    k_model_adam<<<(NP + 255) / 256, 256>>>(m->d_master, m->d_w, m->d_m, m->d_v, m->d_grad, lr, b1t, b2t);
  }
  rc = grad_pass(m, d, k);
  if (rc) return rc;
  float l = 0;
  ACCX_CUDA_TRY(cudaMemcpy(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost));
  if (final_loss) *final_loss = l;
  return ACCX_OK;
}

extern "C" int accx_model_predict(accx_model *m, const float *x, uint32_t k, float *y) {
  if (!m || !x || !y || !k) return ACCX_ERR_INVALID_ARG;
  float *dx = nullptr, *dy = nullptr;
  ACCX_CUDA_TRY(cudaMalloc(&dx, sizeof(float) * (size_t)k * IN));
  cudaError_t e = cudaMalloc(&dy, sizeof(float) * (size_t)k * OUT);
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(float) * (size_t)k * IN, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_model_infer<<<8, 256>>>(m->d_w, dx, k, dy, nullptr, nullptr, accx_kind_bias{});
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(y, dy, sizeof(float) * (size_t)k * OUT, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  if (dy) cudaFree(dy);
  if (e != cudaSuccess) {
    accx_set_cuda_error(e, "model_predict", __FILE__, __LINE__);
    return ACCX_ERR_CUDA;
  }
  return ACCX_OK;
}

static int bucket_stats(accx_graph *g, int mode, uint64_t *edges, double *sum_owner, double *sum_other) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  int rc = ensure_features(g, nullptr, mode);
  if (rc) return rc;
  std::vector<unsigned long long> h(3 * NBB);
  ACCX_CUDA_TRY(cudaMemcpy(h.data(), state_of(g)->d_stats[mode], sizeof(unsigned long long) * 3 * NBB,
                           cudaMemcpyDeviceToHost));
  for (int b = 0; b < NBB; b++) {
    if (edges) edges[b] = h[b];
    if (sum_owner) sum_owner[b] = (double)h[NBB + b];
    if (sum_other) sum_other[b] = (double)h[2 * NBB + b];
  }
  return ACCX_OK;
}

static int bucket_features(accx_graph *g, int mode, float *features) {
  if (!g || !features) return ACCX_ERR_INVALID_ARG;
  int rc = ensure_features(g, nullptr, mode);
  if (rc) return rc;
  ACCX_CUDA_TRY(cudaMemcpy(features, state_of(g)->d_feat[mode], sizeof(float) * NBB * IN, cudaMemcpyDeviceToHost));
  return ACCX_OK;
}

static int model_table_for(accx_model *m, accx_graph *g, int mode, uint8_t *table) {
  if (!m || !g || !table) return ACCX_ERR_INVALID_ARG;
  int rc = ensure_features(g, nullptr, mode);
  if (rc) return rc;
  uint8_t *dt = nullptr;
  ACCX_CUDA_TRY(cudaMalloc(&dt, NBB));
  accx_kind_bias kb;
  for (int o = 0; o < OUT; o++) kb.b[o] = m->bias[o];
  k_model_infer<<<8, 256>>>(m->d_w, state_of(g)->d_feat[mode], NBB, nullptr, state_of(g)->d_stats[mode], dt, kb);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(table, dt, NBB, cudaMemcpyDeviceToHost);
  cudaFree(dt);
  if (e != cudaSuccess) {
    accx_set_cuda_error(e, "model_table_for", __FILE__, __LINE__);
    return ACCX_ERR_CUDA;
  }
  return ACCX_OK;
}

static int set_model(accx_graph *g, int mode, accx_model *m) {
  if (!g) return ACCX_ERR_INVALID_ARG;
  accx_graph_model_state *st = state_of(g);
  if (!st) return ACCX_ERR_OOM;
  st->model[mode] = m;
  return ACCX_OK;
}

extern "C" int accx_bucket_stats(accx_graph *g, uint64_t *edges, double *sum_owner, double *sum_other) {
  return bucket_stats(g, 0, edges, sum_owner, sum_other);
}

extern "C" int accx_model_set_kind_bias(accx_model *m, const float *bias) {
  if (!m || !bias) return ACCX_ERR_INVALID_ARG;
  for (int o = 0; o < OUT; o++) {
    if (!(bias[o] > -1e6f && bias[o] < 1e6f)) return ACCX_ERR_INVALID_ARG;
    m->bias[o] = bias[o];
  }
  return ACCX_OK;
}

extern "C" int accx_model_get_kind_bias(const accx_model *m, float *bias) {
  if (!m || !bias) return ACCX_ERR_INVALID_ARG;
  for (int o = 0; o < OUT; o++) bias[o] = m->bias[o];
  return ACCX_OK;
}
extern "C" int accx_bucket_features(accx_graph *g, float *features) { return bucket_features(g, 0, features); }
extern "C" int accx_model_table_for(accx_model *m, accx_graph *g, uint8_t *table) {
  return model_table_for(m, g, 0, table);
}
extern "C" int accx_graph_set_model(accx_graph *g, accx_model *m) { return set_model(g, 0, m); }

extern "C" int accx_bucket_stats_oriented(accx_graph *g, uint64_t *edges, double *sum_owner, double *sum_other) {
  return bucket_stats(g, 1, edges, sum_owner, sum_other);
}
extern "C" int accx_bucket_features_oriented(accx_graph *g, float *features) {
  return bucket_features(g, 1, features);
}
extern "C" int accx_model_table_for_oriented(accx_model *m, accx_graph *g, uint8_t *table) {
  return model_table_for(m, g, 1, table);
}
extern "C" int accx_graph_set_model_oriented(accx_graph *g, accx_model *m) { return set_model(g, 1, m); }

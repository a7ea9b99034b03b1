// Many graphs in one launch sequence, and the launch autotuner.
//
// A batch joins K graphs into one disjoint-union CSR on the device (vertex ids
// and entry positions shifted by per-graph bases).  Common-neighbour counts,
// similarity, cores, union-find clusters and hubs never cross components, so a
// single count and a single SCAN query over the union give every graph's own
// results (cluster ids shift by the graph's vertex base).  Every counting
// kernel is a persistent grid-stride loop whose work lists live in device
// counters, so the batch's count is a fixed launch sequence: accx_batch_capture
// records it once into a CUDA graph and accx_batch_launch replays it with one
// cudaGraphLaunch.
//
// The autotuner times candidate launch shapes of the bitmap kernel (CTA size,
// dense-window / sparse-table split of its shared memory, i.e. how many chunk
// passes big owners need) on the graph itself and keeps the fastest; it plays
// the role of the reference's num_warps / num_pass command-line knobs
// (scan-query-cuda/experimental/main_scanxp.cpp:24-33).
#include <string.h>

#include <vector>

#include "accx_internal.h"

struct accx_batch_desc {
  const uint32_t *off;
  const int32_t *dst;
  uint32_t n, vbase;
  uint64_t m, ebase;
};

struct accx_batch {
  int k = 0;
  std::vector<uint32_t> vbase, n;
  std::vector<uint64_t> ebase, m;
  accx_graph *u = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

__global__ void k_union(const accx_batch_desc *__restrict__ ds, int k, uint32_t *__restrict__ off,
                        int32_t *__restrict__ dst) {
  for (int gi = blockIdx.y; gi < k; gi += gridDim.y) {
    const accx_batch_desc d = ds[gi];
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < d.m; i += (uint64_t)gridDim.x * blockDim.x)
      dst[d.ebase + i] = d.dst[i] + (int32_t)d.vbase;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < d.n; v += gridDim.x * blockDim.x)
      off[d.vbase + v] = (uint32_t)(d.ebase + d.off[v]);
  }
}

extern "C" int accx_batch_create(accx_graph *const *graphs, int k, void *stream, accx_batch **out) {
  if (!graphs || k < 1 || !out) return ACCX_ERR_INVALID_ARG;
  *out = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  accx_batch *b = new (std::nothrow) accx_batch();
  if (!b) return ACCX_ERR_OOM;
  b->k = k;
  uint64_t N = 0, M = 0;
  bool sym = true;  // the union is symmetric when every member is
  std::vector<accx_batch_desc> ds(k);
  for (int i = 0; i < k; i++) {
    if (!graphs[i]) {
      delete b;
      return ACCX_ERR_INVALID_ARG;
    }
    sym = sym && graphs[i]->symmetric;
    ds[i] = {graphs[i]->d_off, graphs[i]->d_dst, graphs[i]->n, (uint32_t)N, graphs[i]->m, M};
    b->vbase.push_back((uint32_t)N);
    b->n.push_back(graphs[i]->n);
    b->ebase.push_back(M);
    b->m.push_back(graphs[i]->m);
    N += graphs[i]->n;
    M += graphs[i]->m;
  }
  if (N >= 0x7fffffffull || M >= (1ull << 32) - ACCX_DST_PAD) {
    delete b;
    return ACCX_ERR_TOO_LARGE;
  }
  accx_graph *u = new (std::nothrow) accx_graph();
  if (!u) {
    delete b;
    return ACCX_ERR_OOM;
  }
  cudaGetDevice(&u->device);
  u->n = (uint32_t)N;
  u->m = M;
  u->symmetric = sym;
  b->u = u;
  accx_batch_desc *d_ds = nullptr;
  int rc = ACCX_OK;
  do {
    if (accx_dev_alloc((void **)&u->d_off, sizeof(uint32_t) * (N + 1), nullptr) != cudaSuccess ||
        accx_dev_alloc((void **)&u->d_dst, sizeof(int32_t) * (M + ACCX_DST_PAD), nullptr) != cudaSuccess ||
        cudaMalloc(&d_ds, sizeof(accx_batch_desc) * k) != cudaSuccess) { rc = ACCX_ERR_OOM; break; }
    if (cudaMemcpyAsync(d_ds, ds.data(), sizeof(accx_batch_desc) * k, cudaMemcpyHostToDevice, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    uint32_t last = (uint32_t)M;
    if (cudaMemcpyAsync(u->d_off + N, &last, sizeof(uint32_t), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(u->d_dst + M, 0xff, sizeof(int32_t) * ACCX_DST_PAD, s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    dim3 grid(64, k < 65535 ? k : 65535);
    k_union<<<grid, 256, 0, s>>>(d_ds, k, u->d_off, u->d_dst);
    if (cudaGetLastError() != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
    if ((rc = accx_tilerow_build(u, u->d_off, &u->d_tilerow, s)) != ACCX_OK) break;
    if (cudaStreamSynchronize(s) != cudaSuccess) { rc = ACCX_ERR_CUDA; break; }
  } while (0);
  if (d_ds) cudaFree(d_ds);
  if (rc) {
    cudaGetLastError();
    accx_graph_free(u);
    delete b;
    return rc;
  }
  *out = b;
  return ACCX_OK;
}

extern "C" int accx_batch_free(accx_batch *b) {
  if (!b) return ACCX_ERR_INVALID_ARG;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->u) accx_graph_free(b->u);
  delete b;
  return ACCX_OK;
}

extern "C" accx_graph *accx_batch_union(accx_batch *b) { return b ? b->u : nullptr; }

extern "C" int accx_batch_graph_range(const accx_batch *b, int i, uint32_t *vbase, uint32_t *n, uint64_t *ebase,
                                      uint64_t *m) {
  if (!b || i < 0 || i >= b->k) return ACCX_ERR_INVALID_ARG;
  if (vbase) *vbase = b->vbase[i];
  if (n) *n = b->n[i];
  if (ebase) *ebase = b->ebase[i];
  if (m) *m = b->m[i];
  return ACCX_OK;
}

extern "C" int accx_batch_capture(accx_batch *b, const accx_count_opts *opts, void *stream) {
  if (!b) return ACCX_ERR_INVALID_ARG;
  if (opts && (opts->policy == ACCX_POLICY_TABLE || opts->timing)) return ACCX_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (!s) return ACCX_ERR_INVALID_ARG;  // the legacy default stream cannot be captured
  // one eager run allocates every scratch array, so the captured sequence allocates nothing
  int rc = accx_cn_count(b->u, opts, nullptr, stream);
  if (rc) return rc;
  ACCX_CUDA_TRY(cudaStreamSynchronize(s));
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  ACCX_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  rc = accx_cn_count(b->u, opts, nullptr, stream);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) {
    accx_set_cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    return ACCX_ERR_CUDA;
  }
  b->graph = g;
  ACCX_CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
  return ACCX_OK;
}

extern "C" int accx_batch_launch(accx_batch *b, void *stream) {
  if (!b) return ACCX_ERR_INVALID_ARG;
  if (!b->exec) return ACCX_ERR_NOT_READY;
  ACCX_CUDA_TRY(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  return ACCX_OK;
}

// ---------------------------------------------------------------------------
extern "C" int accx_autotune(accx_graph *g, const accx_count_opts *base, int reps, accx_count_opts *best,
                             float *best_ms, float *all_ms, int *ncand, void *stream) {
  if (!g || !best || reps < 1) return ACCX_ERR_INVALID_ARG;
  static const int cands_direct[][3] = {  // block warps, dense KiB, sparse KiB
      {32, 128, 64}, {32, 160, 32}, {32, 96, 96}, {32, 64, 64}, {16, 128, 64}, {16, 48, 32}, {24, 128, 64}};
  // block warps, dense KiB, owner-counter KiB; {0, 0, 0} = the library's default
  // shape (256-thread CTAs, a 24 KiB window)
  static const int cands_orient[][3] = {
      {16, 56, 8}, {16, 48, 16}, {16, 40, 16}, {16, 32, 16}, {32, 64, 16}, {32, 80, 16}, {0, 0, 0}};
  const bool orient = base && base->orient;
  const int(*cands)[3] = orient ? cands_orient : cands_direct;
  const int nc = 7;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  ACCX_CUDA_TRY(cudaEventCreate(&e0));
  ACCX_CUDA_TRY(cudaEventCreate(&e1));
  accx_count_opts o;
  memset(&o, 0, sizeof(o));
  if (base) o = *base;
  o.timing = 0;
  float bms = 1e30f;
  int bi = -1, rc = ACCX_OK;
  for (int c = 0; c < nc && !rc; c++) {
    o.block_warps = cands[c][0];
    o.bitmap_window_kb = cands[c][1];
    o.sparse_table_kb = cands[c][2];
    rc = accx_cn_count(g, &o, nullptr, stream);  // warm (and validates the shape)
    if (rc == ACCX_ERR_INVALID_ARG) {  // shape does not fit this device: skip it
      rc = ACCX_OK;
      if (all_ms) all_ms[c] = -1.f;
      continue;
    }
    if (rc) break;
    float ms = 1e30f;
    for (int r = 0; r < reps && !rc; r++) {
      cudaEventRecord(e0, s);
      rc = accx_cn_count(g, &o, nullptr, stream);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      ms = t < ms ? t : ms;
    }
    if (all_ms) all_ms[c] = ms;
    if (ms < bms) {
      bms = ms;
      bi = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (ncand) *ncand = nc;
  if (bi < 0) return ACCX_ERR_INVALID_ARG;
  o.block_warps = cands[bi][0];
  o.bitmap_window_kb = cands[bi][1];
  o.sparse_table_kb = cands[bi][2];
  *best = o;
  if (best_ms) *best_ms = bms;
  return ACCX_OK;
}

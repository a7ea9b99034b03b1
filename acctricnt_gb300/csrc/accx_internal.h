// Internal definitions shared by the libaccx translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>

#include "../../include/accx.h"

#define ACCX_VERSION_STR "accx 0.1 sm_103a"

// Device arrays are padded by this many int32 so that 16-byte vector loads of
// a list's last window never leave the allocation.
#define ACCX_DST_PAD 64

// Scratch and results of one SCAN query; a graph handle owns one, and
// accx_query_ctx_create makes more so that several queries can run on the same
// resident graph at once (each on its own stream).
struct accx_query_ctx {
  uint32_t *d_simbits = nullptr;  // ceil(m/32) words
  int32_t *d_core_count = nullptr;
  int32_t *d_label = nullptr;
  int32_t *d_parent = nullptr;
  int32_t *d_hubmin = nullptr;
  int32_t *d_hubmax = nullptr;
  unsigned long long *d_qcounters = nullptr;  // query counters
  uint32_t *d_corebits = nullptr;             // n bits: core flags of the last query
  uint32_t *d_big = nullptr;                  // vertices whose rows are counted by a whole CTA
  bool query_valid = false;
  double last_eps = 0;
  int last_mu = 0;
  // pairs of the last query (built on demand)
  unsigned long long *d_pairs = nullptr;
  unsigned long long *d_pairs_tmp = nullptr;
  uint64_t pairs_cap = 0;
  uint64_t npairs = 0;
  bool pairs_valid = false;
  accx_scan_summary summary{};
  uint32_t n = 0;   // sizes the arrays were made for
  uint64_t m = 0;
};
void accx_query_ctx_release(accx_query_ctx *q);

struct accx_graph {
  int device = 0;
  // stream the handle was made on: when set, its device arrays come from and
  // return to the stream-ordered allocator on it (no device-wide sync on free)
  cudaStream_t home = nullptr;
  uint32_t n = 0;
  uint64_t m = 0;
  uint32_t *d_off = nullptr;  // n+1
  int32_t *d_dst = nullptr;   // m + ACCX_DST_PAD
  int32_t *d_cnt = nullptr;   // m
  float *d_simkey = nullptr;    // m: similarity key per entry (built by the first query after a count)
  uint32_t *d_src = nullptr;    // m: source vertex (row) of every entry, built with the keys
  // set (release) once d_simkey/d_src hold the keys of the current counts; query
  // threads read it (acquire) before using those arrays without the key lock
  std::atomic<bool> key_valid{false};
  uint32_t *d_tilerow = nullptr;   // row of every 256-entry tile's first entry (+1 for the last entry)
  uint32_t *d_rtilerow = nullptr;  // the same for the relabeled CSR
  // degree-descending relabel (accx_graph_relabel): counting runs on these
  uint32_t *d_roff = nullptr;   // n+1
  int32_t *d_rdst = nullptr;    // m + ACCX_DST_PAD
  uint32_t *d_rmap = nullptr;   // m: original entry -> relabeled entry
  int32_t *d_rcnt = nullptr;    // m: counts in relabeled order
  uint32_t *d_oldid = nullptr;  // n: new id -> original id
  uint32_t *d_newid = nullptr;  // n: original id -> new id
  int32_t cnt_bias = 0;
  bool cnt_valid = false;

  // counting scratch
  uint2 *d_edge_list = nullptr;  // m/2+1 owned entries: merge items from the front, gallop from the back
  unsigned long long *d_icnt = nullptr;    // n+1 bitmap items per owner
  unsigned long long *d_prefix = nullptr;  // n+1 exclusive prefix of d_icnt
  uint32_t *d_pre = nullptr;               // n prefix lengths (neighbours with smaller ids), oriented counts
  uint2 *d_vinfo = nullptr;                // n (offset, prefix length) of the counting CSR, oriented counts
  uint2 *d_or_sl = nullptr;                // m oriented bitmap entries: (partner prefix start, cut length), 0 length = not bitmap
  uint32_t *d_or_items = nullptr;          // n + m/32 + 1 oriented bitmap work items: owner of each
  uint32_t *d_rev = nullptr;               // m reverse entry of every entry of the counting CSR (oriented counts)
  uint32_t *d_rev_orig = nullptr;          // m reverse entries of the handle's own CSR, recorded by full validation
  bool symmetric = false;                  // known symmetric: validated, generated or built from an edge list
  const uint32_t *rev_csr = nullptr;       // the offsets array d_rev was built for
  void *d_scan_tmp = nullptr;
  size_t scan_tmp_bytes = 0;
  unsigned long long *d_counters = nullptr;  // [0] merge, [1] gallop, [2] bitmap items, [3..5] work per kind
  uint64_t stats_edges[ACCX_NUM_KINDS] = {0, 0, 0};
  uint64_t stats_work[ACCX_NUM_KINDS] = {0, 0, 0};
  uint8_t *d_table = nullptr;  // ACCX_NB*ACCX_NB kinds
  cudaEvent_t ev[ACCX_NUM_PHASES + 1] = {};
  bool timed = false;

  // SCAN query state of the handle's own queries (accx_scan_query)
  accx_query_ctx qc;

  // trained cost model state (accx_model_*)
  void *model = nullptr;
};

#define ACCX_CUDA_TRY(call)                                   \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) {                                  \
      accx_set_cuda_error(_e, #call, __FILE__, __LINE__);     \
      return (_e == cudaErrorMemoryAllocation) ? ACCX_ERR_OOM \
                                               : ACCX_ERR_CUDA; \
    }                                                         \
  } while (0)

void accx_set_cuda_error(cudaError_t e, const char *what, const char *file, int line);

// Device memory on a stream's pool when s != NULL (no device-wide synchronisation
// on free), else plain cudaMalloc/cudaFree.
cudaError_t accx_dev_alloc(void **p, size_t bytes, cudaStream_t s);
void accx_dev_free(void *p, cudaStream_t s);

// True when p is a device (or managed) pointer.
bool accx_is_device_ptr(const void *p);

// Copies between host/device buffers chosen by pointer kind.
int accx_copy_out(void *dst, const void *dev_src, size_t bytes, cudaStream_t s);
int accx_copy_in(void *dev_dst, const void *src, size_t bytes, cudaStream_t s);

// Grid for a grid-stride kernel: enough CTAs to fill every SM `per_sm` times.
int accx_grid_for(int device, int block, int per_sm);
int accx_sm_count(int device);

// Internal: creates a handle around device arrays already owned by it.
int accx_graph_validate_device(accx_graph *g, int full, int exact, cudaStream_t s);
int accx_ensure_count_scratch(accx_graph *g);
// Prefix lengths (neighbours with smaller ids) of the CSR counts run on (the
// relabeled copy when there is one) into g->d_pre (count.cu).
int accx_prefix_lengths(accx_graph *g, cudaStream_t s);

// Cost-model state attached to a handle (model.cu); orient selects the direct
// (0) or oriented (1) buckets, features and attached model.
void accx_model_release(accx_graph *g);
int accx_model_table(accx_graph *g, uint8_t *table);
int accx_model_table_device(accx_graph *g, cudaStream_t s, int orient);
// Predicted time (ms) of a model's own table on a graph's buckets (direct: mode 0,
// oriented: mode 1), computed on the device.
int accx_model_plan_ms(accx_model *m, accx_graph *g, int mode, cudaStream_t s, double *ms);

// Exclusive/inclusive helpers implemented in gen.cu.
// Row index of every 256-entry tile of a CSR (graph.cu), allocated on g's home stream.
int accx_tilerow_build(accx_graph *g, const uint32_t *off, uint32_t **out, cudaStream_t s);
// Reverse index of g's CSR (off, tilerow, dst) by a stable sort of the entries
// by neighbour id; with d_status the symmetry it relies on is checked (graph.cu).
int accx_rev_by_sort(accx_graph *g, const uint32_t *off, const uint32_t *tilerow, const int32_t *dst, int *d_status,
                     cudaStream_t s, uint32_t **rev_out);

// Relabeled counts -> the handle's entry order (relabel.cu).
int accx_relabel_gather(accx_graph *g, int32_t *host, cudaStream_t s);
// The device address of pinned (mapped) host memory, or nullptr (graph.cu).
void *accx_mapped_host(const void *p);

int accx_build_csr_from_keys(accx_graph *g, unsigned long long *d_keys, uint64_t nkeys, uint32_t n,
                             cudaStream_t s);

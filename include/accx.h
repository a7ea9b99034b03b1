/*
 * accx.h -- C ABI of the GB300-native all-edge common-neighbour (CN) counter and
 * SCAN structural-clustering query (libaccx.so).
 *
 * Every function returns ACCX_OK (0) or a negative status (see accx_strerror);
 * nothing in the library calls exit() or traps.  Pointers are plain host or
 * device pointers; "stream" is a cudaStream_t passed as void* (NULL = the legacy
 * default stream).  A graph handle is not thread-safe: use one handle per thread,
 * or serialise calls on it.
 *
 * Reference interfaces replaced (paths inside the AccTriCnt tree):
 *   accx_graph_create / accx_graph_load_dir
 *       Graph::Graph, ReadDegree, ReadAdjacencyList, CheckInputGraph
 *       (scan-query-cuda/util/graph.cu:33-51, :53-70, :76-194, :196-214)
 *   accx_cn_count
 *       SCAN_XP::CheckCore (scan-query-cuda/experimental_scan_xp_multigpu_multipass.cu:3-166):
 *       kernels set_intersection_GPU_bitmap_warp_per_vertex, _shared_merge_filtered,
 *       _shared_galloping_filtered (scan-query-cuda/scan_xp_multi_gpu_multi_pass_common.cu:32-495)
 *       and the reverse-offset mirror (PostComputeCoreChecking, scan-query-cuda/scan_xp_common.cu:220-237)
 *   accx_scan_query
 *       PostComputeCoreChecking similarity/core part (scan_xp_common.cu:239-267),
 *       ClusterCore (:73-85), LabelNonCore/CheckHub (:87-111), PostProcess (:113-135),
 *       MarkClusterMinEleAsId (:137-158)
 *   accx_scan_pairs / accx_write_result
 *       PrepareResultOutput (scan_xp_common.cu:160-199) and Graph::Output (util/graph.cu:216-245)
 */
#ifndef ACCX_H
#define ACCX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define ACCX_OK 0
#define ACCX_ERR_INVALID_ARG (-1)   /* NULL handle/pointer, bad size or option */
#define ACCX_ERR_CUDA (-2)          /* a CUDA runtime call failed */
#define ACCX_ERR_OOM (-3)           /* device or host allocation failed */
#define ACCX_ERR_SELF_LOOP (-4)     /* input has an entry (u,u) */
#define ACCX_ERR_UNSORTED (-5)      /* a neighbour list is not strictly increasing */
#define ACCX_ERR_RANGE (-6)         /* a neighbour id >= n, or offsets inconsistent */
#define ACCX_ERR_ASYMMETRIC (-7)    /* (u,v) present without (v,u) */
#define ACCX_ERR_IO (-8)            /* a graph or result file cannot be read/written */
#define ACCX_ERR_TOO_LARGE (-9)     /* sizes beyond the format (m >= 2^32) or a stated limit */
#define ACCX_ERR_NOT_READY (-10)    /* counts not computed yet, or request still running */
#define ACCX_ERR_TIMEOUT (-11)      /* a bounded device wait gave up */
#define ACCX_ERR_ADMISSION (-12)    /* a request does not fit the server's HBM budget */
#define ACCX_ERR_NO_DEVICE (-13)    /* no CUDA device visible */

const char *accx_strerror(int status);

/* Library build identification ("accx <version> sm_103a"). */
const char *accx_version(void);

/* ---- graphs ---------------------------------------------------------------- */
typedef struct accx_graph accx_graph;

/* Flags for accx_graph_create. */
#define ACCX_GRAPH_VALIDATE 1u       /* check self loops, order, range, symmetry on the GPU */
/* With ACCX_GRAPH_VALIDATE, how symmetry is checked.  By default in the same pass
 * as the other checks, by two 64-bit multiset fingerprints (the sums over all
 * entries (u,v) of two mixing functions of (u,v), against the same sums of (v,u));
 * rows are already checked strictly increasing, so an asymmetric graph passes
 * only if both 64-bit sums collide.  ACCX_GRAPH_VALIDATE_EXACT instead sorts the
 * entries by neighbour id (about 16 bytes per entry of scratch, several times the
 * time) and records the reverse index on the way. */
#define ACCX_GRAPH_VALIDATE_EXACT 2u

/* Copies a CSR (off[n+1], dst[m], host or device pointers -- detected with
 * cudaPointerGetAttributes) to device memory and returns a handle.  dst holds
 * sorted neighbour ids without self loops, as the reference's b_adj.bin. */
int accx_graph_create(const uint32_t *off, const int32_t *dst, uint32_t n, uint64_t m, unsigned flags,
                      void *stream, accx_graph **out);

/* Reads <dir>/b_degree.bin and <dir>/b_adj.bin (the reference format: int32
 * int_size, uint32 n, uint32 m, int32 degree[n]; int32 dst[m]) straight into a
 * handle.  Validates like Graph::CheckInputGraph. */
int accx_graph_load_dir(const char *dir, unsigned flags, void *stream, accx_graph **out);

int accx_graph_free(accx_graph *g);
int accx_graph_size(const accx_graph *g, uint32_t *n, uint64_t *m);

/* Builds (once) a degree-descending relabeled copy of the CSR on the device,
 * the GPU form of the reference's "deg" reorder (scan-query/scan_xp.cpp:1145-1222,
 * :1279-1301).  Later counts run on it and are mapped back to the handle's entry
 * order, so results are unchanged; the shared-memory bitmap then serves most
 * probes from its dense low-id window.  Costs 4*(n+1) + 12*m bytes of HBM. */
int accx_graph_relabel(accx_graph *g, void *stream);
int accx_graph_is_relabeled(const accx_graph *g);

/* Copies the relabeled CSR and its maps out (host or device pointers; any may
 * be NULL): roff[n+1], rdst[m], map[m] (original entry -> relabeled entry),
 * oldid[n] (new id -> original id).  ACCX_ERR_NOT_READY before accx_graph_relabel.
 * No reference counterpart: the reference keeps its reorder maps internal
 * (scan-query/util/graph.cpp:176-216). */
int accx_graph_relabeled_csr(const accx_graph *g, uint32_t *roff, int32_t *rdst, uint32_t *map, uint32_t *oldid,
                             void *stream);

/* Copies the CSR back (host or device destination pointers). */
int accx_graph_download(const accx_graph *g, uint32_t *off, int32_t *dst, void *stream);

/* Device pointers of the resident arrays (off[n+1], dst[m padded], cnt[m] or
 * NULL before the first count).  Valid until accx_graph_free. */
int accx_graph_device_ptrs(const accx_graph *g, const uint32_t **off, const int32_t **dst, const int32_t **cnt);

/* Device-side synthetic generators (seeded, counter-based: the same seed gives the
 * same graph on any GPU and on the host generator below).  The edge stream is
 * symmetrised; self loops and duplicate edges are removed; lists are sorted. */
#define ACCX_GEN_RMAT 0      /* p0 = scale, p1 = edge factor, a,b,c in q0..q2 */
#define ACCX_GEN_ER 1        /* p0 = n, p1 = undirected edge draws (n*mean/2) */
#define ACCX_GEN_CHUNG_LU 2  /* p0 = n, p1 = edge draws, q0 = gamma, q1 = max expected degree */
typedef struct {
  int kind;
  uint64_t p0, p1;
  double q0, q1, q2;
  uint64_t seed;
} accx_gen_params;

/* A handle generated on a non-NULL stream takes its device arrays from that
 * stream's memory pool and returns them there on accx_graph_free (no device-wide
 * synchronisation); keep that stream alive until the handle is freed. */
int accx_graph_generate(const accx_gen_params *params, void *stream, accx_graph **out);

/* Host generator with the same output, for tests and for files.  Two calls:
 * with off/dst NULL it returns the sizes; then fill caller buffers of n+1 / m. */
int accx_generate_host(const accx_gen_params *params, uint32_t *n, uint64_t *m, uint32_t *off, int32_t *dst);

/* Builds a graph from an undirected edge list on the device, as the
 * reference's EdgeListToBinsConverter does on the host
 * (scan-query/converter/EdgeListToBinsConverter.cpp:24-126): both directions of
 * every (src[i], dst[i]) are kept, self loops and duplicates dropped, lists
 * sorted.  n = number of vertices (ids must be < n); src/dst host or device. */
int accx_graph_from_edges(const uint32_t *src, const uint32_t *dst, uint64_t k, uint32_t n, void *stream,
                          accx_graph **out);

/* Triangles of the graph from its resident counts: sum of all counts / 6
 * (every triangle adds one common neighbour to each of its 3 edges, both
 * directions).  Needs a count (any bias; the bias is removed). */
int accx_triangles(const accx_graph *g, uint64_t *triangles, void *stream);

/* Count persistence: writes the resident counts (int32 per entry, the bias
 * included) with a header of n, m and bias to `path`, and reads them back into
 * a handle of the same graph, so a restarted server need not recount. */
int accx_cn_save(const accx_graph *g, const char *path);
int accx_cn_load(accx_graph *g, const char *path);

/* Splits [0, n) into `parts` vertex ranges of equal filtered cost, cost(u) =
 * sum over v in N(u), v > u of (deg v + 2) -- the reference's multi-GPU
 * partitioner ComputeVertexRangeAccumulatedFilteredDegree
 * (scan-query-cuda/scan_xp_multi_gpu_multi_pass_common.cu:516-554), computed on
 * the device.  ranges[parts+1]: ranges[0] = 0, ranges[parts] = n. */
int accx_vertex_ranges(const accx_graph *g, int parts, uint32_t *ranges, void *stream);

/* Writes a CSR in the reference's b_degree.bin / b_adj.bin format. */
int accx_write_graph_dir(const char *dir, const uint32_t *off, const int32_t *dst, uint32_t n, uint64_t m);

/* ---- all-edge CN counting ---------------------------------------------------- */
/* Kernel kinds a policy can assign to a degree bucket. */
#define ACCX_KIND_MERGE 0   /* warp merge-path over uint4-vectorised windows */
#define ACCX_KIND_GALLOP 1  /* per-element binary search of the small list in the large one */
#define ACCX_KIND_BITMAP 2  /* per-owner shared-memory bitmap over id windows, ballot/popc probe */
#define ACCX_NUM_KINDS 3
#define ACCX_KIND_SKIP 3    /* table only: leave the bucket uncounted (per-bucket timing runs) */

/* Policies. */
#define ACCX_POLICY_HEURISTIC 0 /* reference rule: gallop iff d_max/50 > d_min, else merge */
#define ACCX_POLICY_TABLE 1     /* per-bucket kinds from `table` (ACCX_NB x ACCX_NB bytes) */
#define ACCX_POLICY_MERGE 2     /* every edge by one kind ... */
#define ACCX_POLICY_GALLOP 3
#define ACCX_POLICY_BITMAP 4
#define ACCX_POLICY_MODEL 5     /* the handle's trained cost model (accx_model_*) picks per bucket */

/* Degree buckets: b(d) = min(floor(log2 d), ACCX_NB-1) for d >= 1.  An edge's
 * bucket is (b(d_owner), b(d_other)); the owner is the endpoint with the larger
 * degree (ties: smaller id), as in the reference CPU bitmap build. */
#define ACCX_NB 24

typedef struct {
  int policy;
  const uint8_t *table;   /* ACCX_NB*ACCX_NB kinds, row = owner bucket; for ACCX_POLICY_TABLE */
  int32_t bias;           /* added to every count; 2 gives the reference's common_node_num */
  int block_warps;        /* bitmap/merge CTA size in warps (0 = tuned default) */
  int bitmap_window_kb;   /* dense shared-memory bitmap over the lowest ids, KiB (0 = tuned default) */
  int timing;             /* 1: record CUDA events around each phase (accx_cn_last_timings) */
  int sparse_table_kb;    /* hashed bitmap-word table for the other ids, KiB (0 = tuned default) */
  int sm_limit;           /* run the persistent counting kernels on at most this many SMs (0 = all);
                             leaves SMs free for latency-critical work on other streams */
  int orient;             /* 0: direct -- every owned edge intersects the two full lists.
                             1: oriented -- |N(u) ∩ N(v)| is the number of triangles on (u,v); each
                             triangle a<b<c is found once, from the edge (c,b), by intersecting the
                             prefix lists N(c) ∩ [0,b) and N(b) ∩ [0,b), and credited to its three
                             edges.  Edge owners, buckets and kinds then use prefix lengths (neighbours
                             with smaller ids) instead of degrees.  Exact either way; oriented does far
                             less work on a degree-descending relabeled graph (accx_graph_relabel),
                             where prefix lists hold at most sqrt(2m) ids.  ACCX_POLICY_MODEL then uses
                             the model attached by accx_graph_set_model_oriented. */
} accx_count_opts;

/* Counts cnt[e] = |N(u) ∩ N(v)| + bias for every CSR entry e=(u,v) into the
 * handle's resident count array, then (if out != NULL) copies it to `out` (host
 * or device).  opts NULL = heuristic policy, bias 0. */
int accx_cn_count(accx_graph *g, const accx_count_opts *opts, int32_t *out, void *stream);

/* Copies the resident counts of the last count (or captured replay) to `out`
 * (host or device), without counting again. */
int accx_cn_read(const accx_graph *g, int32_t *out, void *stream);

/* Sum of the resident counts and an order-independent hash of every
 * (entry, count) pair: a compact fingerprint for comparing two count runs. */
int accx_cn_digest(const accx_graph *g, uint64_t *sum, uint64_t *digest, void *stream);

/* Per-kind statistics of the last accx_cn_count: edges[k] owned edges and
 * work[k] probe elements assigned to kind k. */
int accx_cn_last_stats(const accx_graph *g, uint64_t edges[ACCX_NUM_KINDS], uint64_t work[ACCX_NUM_KINDS]);

/* Owner-side elements per kind of the last count: sum of owner degrees over the
 * merge/gallop edges, and the owner lists the bitmap kernel staged (per work item). */
int accx_cn_last_owner_work(const accx_graph *g, uint64_t owner_work[ACCX_NUM_KINDS]);

/* Oriented counts: common ids found per kind (each a triangle) in the last
 * count, and the ids the bitmap kind actually probed (partner prefixes after the
 * cut at the smaller id).  Zero after a direct count. */
int accx_cn_last_matches(const accx_graph *g, uint64_t matches[ACCX_NUM_KINDS], uint64_t *probed);

/* Phases timed when accx_count_opts.timing is set. */
#define ACCX_PHASE_PLAN 0    /* classify + bitmap work items */
#define ACCX_PHASE_MERGE 1
#define ACCX_PHASE_GALLOP 2
#define ACCX_PHASE_BITMAP 3
#define ACCX_PHASE_MIRROR 4
#define ACCX_NUM_PHASES 5
/* Milliseconds per phase of the last timed count (waits for it to finish). */
int accx_cn_last_timings(const accx_graph *g, float ms[ACCX_NUM_PHASES]);

/* All-edge counts without allocating any memory.  (No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc -- a plugin in a
 * process whose framework owns every byte of device memory, code under a
 * stream-ordered pool budget, or a loop that must never enter the driver's
 * allocator.)  off/dst/cnt are device pointers: a symmetric CSR as
 * accx_graph_create accepts it, and the int32 output, cnt[e] = |N(u) ∩ N(v)| +
 * bias for every entry.  Precondition: the CSR is symmetric, sorted and free of
 * self loops (validate it once with accx_graph_create and ACCX_GRAPH_VALIDATE);
 * this call does not check it, and on an asymmetric CSR some entries of cnt are
 * left unspecified while the call still returns ACCX_OK.  The only scratch is a fixed 8 MiB array inside the
 * library that every GPU loading the library keeps until the process exits, so
 * graphs are limited to accx_cn_count_noalloc_max_entries() CSR entries (2^21);
 * larger ones get ACCX_ERR_TOO_LARGE, host pointers ACCX_ERR_INVALID_ARG.  The
 * first call on a device looks up that array's device address (make it before
 * any stream capture on that device).  All calls share the array: calls that
 * overlap on the GPU (other streams, other threads) race and must be ordered by
 * the caller. */
int accx_cn_count_noalloc(const uint32_t *off, const int32_t *dst, uint32_t n, uint64_t m, int32_t bias,
                          int32_t *cnt, void *stream);
uint64_t accx_cn_count_noalloc_max_entries(void);

/* ---- learned scheduler: an MLP cost model per degree bucket ------------------
 * No counterpart in the reference, which fixes the kernel choice by a degree
 * ratio (scan_xp_multi_gpu_multi_pass_common.cu:57-59, :105-117).  The model maps
 * a bucket's features (owner/other mean degree, their ratio, bucket size, graph
 * size; ACCX_MODEL_IN floats) to the predicted log2 time per edge of each kernel
 * kind; the scheduler picks the cheapest kind per bucket.  Weights are FP16,
 * accumulation FP32; training, inference and the gradient run as the library's
 * own CUDA kernels. */
#define ACCX_MODEL_IN 8
#define ACCX_MODEL_H 32
#define ACCX_MODEL_OUT ACCX_NUM_KINDS
#define ACCX_MODEL_NPARAMS (ACCX_MODEL_IN * ACCX_MODEL_H + ACCX_MODEL_H + ACCX_MODEL_H * ACCX_MODEL_H + ACCX_MODEL_H + \
                            ACCX_MODEL_H * ACCX_MODEL_OUT + ACCX_MODEL_OUT)
typedef struct accx_model accx_model;

int accx_model_create(uint64_t seed, accx_model **out);
int accx_model_free(accx_model *m);
/* Parameters as FP32 (the FP16 weights widened); set rounds them to FP16. */
int accx_model_get_params(const accx_model *m, float *params);
int accx_model_set_params(accx_model *m, const float *params);
/* Per-bucket statistics of a graph's owned edges: edges[b], and the sums of the
 * owner's and the other endpoint's degree, b = owner_bucket*ACCX_NB + other_bucket. */
int accx_bucket_stats(accx_graph *g, uint64_t *edges, double *sum_owner, double *sum_other);
/* Feature rows (ACCX_MODEL_IN floats per bucket, ACCX_NB*ACCX_NB rows) of a graph. */
int accx_bucket_features(accx_graph *g, float *features);
/* Mean loss and its gradient (FP32, ACCX_MODEL_NPARAMS) over k samples:
 * x[k*ACCX_MODEL_IN], kind[k], target[k] (log2 seconds per edge). */
int accx_model_loss_grad(accx_model *m, const float *x, const int32_t *kind, const float *target, uint32_t k,
                         float *grad, float *loss);
/* Adam training on the GPU over the samples; returns the final mean loss. */
int accx_model_train(accx_model *m, const float *x, const int32_t *kind, const float *target, uint32_t k,
                     int epochs, float lr, float *final_loss);
/* Predictions (log2 seconds per edge, ACCX_MODEL_OUT per row) for k feature rows. */
int accx_model_predict(accx_model *m, const float *x, uint32_t k, float *y);
/* The kind table the model picks for a graph (runs on the device): per bucket
 * the kind with the smallest prediction + kind bias. */
int accx_model_table_for(accx_model *m, accx_graph *g, uint8_t *table);
/* Per-kind log2 offsets added to the predictions before a table's argmin
 * (default 0).  Per-bucket timings taken with the other buckets skipped
 * overstate the bitmap kind, whose owner staging serves all of an owner's
 * buckets; the scheduler fits this offset on whole-count timings. */
int accx_model_set_kind_bias(accx_model *m, const float *bias);
int accx_model_get_kind_bias(const accx_model *m, float *bias);
/* Attach a model to a graph handle for ACCX_POLICY_MODEL (the handle does not own it). */
int accx_graph_set_model(accx_graph *g, accx_model *m);
/* The same for oriented counts (accx_count_opts.orient = 1): buckets by prefix
 * length (owner = longer prefix; edges whose shorter prefix is empty left out) on
 * the CSR counts run on -- the relabeled copy when there is one.  The oriented
 * kernels have their own costs, so they get their own model. */
int accx_bucket_stats_oriented(accx_graph *g, uint64_t *edges, double *sum_owner, double *sum_other);
int accx_bucket_features_oriented(accx_graph *g, float *features);
int accx_model_table_for_oriented(accx_model *m, accx_graph *g, uint8_t *table);
int accx_graph_set_model_oriented(accx_graph *g, accx_model *m);

/* ---- scheduler: training data, training, calibration, count plan, model file --
 * Replaces the reference's fixed kernel choice: the backend linked into each
 * CMake target (scan-query-cuda/CMakeLists.txt:114-117, each target defining its
 * own SCAN_XP::CheckCore) and the ratio-50 rule inside it
 * (scan_xp_multi_gpu_multi_pass_common.cu:57-59, :105-117), which stays the
 * fallback when no model is available.  A scheduler holds two cost models, one
 * for the direct kernels and one for the oriented kernels.  It is not
 * thread-safe: a tuned plan changes its models' bitmap offsets. */

/* Per-bucket kernel timings of a graph, the models' training data: for every
 * bucket with at least min_edges owned edges and every kind k, one count with
 * only that bucket enabled under kind k (all others ACCX_KIND_SKIP), best of
 * reps; ms[b*ACCX_NUM_KINDS + k] = its counting-phase time minus that of a count
 * with every bucket skipped (NaN for buckets not timed).  edges[b] as
 * accx_bucket_stats (accx_bucket_stats_oriented when orient = 1). */
int accx_bucket_timings(accx_graph *g, int orient, int reps, uint64_t min_edges, uint64_t *edges, float *ms,
                        void *stream);

#define ACCX_SCHED_NOFFSETS 10  /* bitmap-kind log2 offsets tried: 0, -0.5, -1, -1.5, -2, -3, -5, -64
                                   (-64: the bitmap kind for every bucket), 1, 64 (never the bitmap kind) */
typedef struct accx_sched accx_sched;
typedef struct {
  uint64_t seed;  /* model initialisation (0 = 1) */
  int epochs;     /* Adam epochs per model (0 = 4000; 800 when quick) */
  float lr;       /* learning rate (0 = 3e-3) */
  int reps;       /* timing repetitions per bucket and kind (0 = 2) */
  int quick;      /* 1: four small training graphs, also used for calibration (tests) */
  int candidates; /* models trained per mode (seeds seed, seed+1, ...) on the same rows; the
                     calibration keeps the best (0 = 3; 1 when quick; at most
                     ACCX_SCHED_MAX_CANDIDATES) */
} accx_sched_config;
#define ACCX_SCHED_MAX_CANDIDATES 8
typedef struct {
  uint32_t rows[2];                   /* training rows per model (0 direct, 1 oriented) */
  float loss_initial[2], loss_final[2];
  float bitmap_offset[2];             /* the calibrated log2 offset of the bitmap kind */
  float calib_relative[2][ACCX_SCHED_NOFFSETS];  /* size-weighted relative count time per offset */
  double collect_s[2], train_s[2], calibrate_s[2];
  int quick;
  int candidates[2];                  /* models trained per mode */
  int chosen[2];                      /* the candidate kept */
  float candidate_score[2][ACCX_SCHED_MAX_CANDIDATES];  /* each one's best calibration score
                                                           (relative to the best count per graph) */
} accx_sched_info;
typedef struct {
  int orient;                 /* the chosen mode */
  double predicted_ms[2];     /* each model's predicted time of its own table (direct, oriented) */
  float calibrated_offset;    /* the chosen mode's bitmap offset before tuning */
  float bitmap_offset;        /* ... and after */
  int tuned;
  float offsets[ACCX_SCHED_NOFFSETS];
  float tune_ms[ACCX_SCHED_NOFFSETS];  /* whole-count time per candidate offset (tuned only) */
  double tune_s;
  double mode_ms[2];          /* tuned only: each mode's own table as a whole count (direct, oriented) */
} accx_sched_plan;

/* Trains both models on the device: per-bucket timings of seven seeded graphs
 * (relabeled), Adam training with the library's kernels of several candidate
 * models (different seeds, the same rows), then the candidate and its bitmap
 * offset chosen on whole counts of those graphs plus R-MAT 20 and 22.
 * Takes tens of seconds on a GB300 (a few with quick = 1).  cfg NULL = defaults. */
int accx_sched_train(const accx_sched_config *cfg, accx_sched **out);
int accx_sched_free(accx_sched *s);
/* A text file of both models (parameters, kind offsets, training record). */
int accx_sched_save(const accx_sched *s, const char *path);
int accx_sched_load(const char *path, accx_sched **out);
int accx_sched_get_info(const accx_sched *s, accx_sched_info *info);
/* The scheduler's model for a mode (owned by the scheduler). */
int accx_sched_model(accx_sched *s, int orient, accx_model **out);
/* Plans the counts of g: attaches both models (ACCX_POLICY_MODEL), predicts each
 * mode's time from its own per-bucket table and picks the faster mode.  tune = 1
 * instead picks the mode by measurement (each mode's table as a whole count),
 * then times one whole count per bitmap offset on g and keeps the fastest in the
 * chosen model (it then applies to every graph that model serves).  opts
 * (optional) is filled for accx_cn_count: policy ACCX_POLICY_MODEL, orient. */
int accx_sched_plan_for(accx_sched *s, accx_graph *g, int tune, accx_count_opts *opts, accx_sched_plan *plan,
                        void *stream);

/* ---- batches of uneven graphs -------------------------------------------------
 * No reference counterpart (the reference counts one graph per process).  A
 * batch joins K graphs into one disjoint-union CSR on the device; one count and
 * one SCAN query over the union give each graph's results (graph i owns vertex
 * ids [vbase_i, vbase_i + n_i) and entries [ebase_i, ebase_i + m_i); cluster ids
 * are union ids).  The count is a fixed launch sequence of persistent kernels,
 * recorded once into a CUDA graph by accx_batch_capture and replayed by
 * accx_batch_launch. */
typedef struct accx_batch accx_batch;
int accx_batch_create(accx_graph *const *graphs, int k, void *stream, accx_batch **out);
int accx_batch_free(accx_batch *b);
/* The union graph (owned by the batch): count, relabel, query and download it
 * with the accx_graph functions. */
accx_graph *accx_batch_union(accx_batch *b);
int accx_batch_graph_range(const accx_batch *b, int i, uint32_t *vbase, uint32_t *n, uint64_t *ebase, uint64_t *m);
/* Records the count of the union (opts as for accx_cn_count, not ACCX_POLICY_TABLE
 * and without timing) on `stream` (not the legacy default stream); runs it once
 * eagerly first so every scratch array exists before capture. */
int accx_batch_capture(accx_batch *b, const accx_count_opts *opts, void *stream);
int accx_batch_launch(accx_batch *b, void *stream);

/* Launch autotuner: times candidate shapes of the bitmap kernel (CTA warps,
 * dense-window KiB, sparse-table KiB) for a policy on this graph and returns the
 * fastest in *best (other fields copied from *base).  all_ms (optional, >= 8
 * floats) receives each candidate's time, -1 for shapes the device cannot run.
 * For oriented counts one candidate is the default shape (all three 0). */
int accx_autotune(accx_graph *g, const accx_count_opts *base, int reps, accx_count_opts *best, float *best_ms,
                  float *all_ms, int *ncand, void *stream);

/* ---- SCAN query ------------------------------------------------------------- */
#define ACCX_UNCLASSIFIED 0
#define ACCX_CORE 1
#define ACCX_HUB 2

typedef struct {
  uint32_t cores, clusters, hubs, outliers; /* PostProcess counts */
  uint64_t similar_entries;                 /* entries with sim = 1 */
  uint64_t noncore_pairs;                   /* unique (cluster, non-core) pairs */
  uint64_t digest;                          /* order-independent hash of every (vertex, label, cluster) */
} accx_scan_summary;

/* Runs the SCAN query on the resident counts (accx_cn_count must have run with
 * any bias; the bias is taken into account).  Outputs are optional (NULL =
 * skip, host or device pointers): sim[m] (0/1 bytes), label[n] (0/1/2),
 * cluster[n] (minimum vertex id of the core's cluster, -1 for non-cores). */
int accx_scan_query(accx_graph *g, double eps, int mu, uint8_t *sim, int32_t *label, int32_t *cluster,
                    accx_scan_summary *summary, void *stream);

/* Query contexts: the scratch and results of one query.  accx_scan_query uses
 * the handle's own context; with extra contexts several queries can run on one
 * resident graph at the same time, each on its own stream (the graph and its
 * counts are only read).  A context is sized for one graph. */
typedef struct accx_query_ctx accx_query_ctx;
int accx_query_ctx_create(const accx_graph *g, accx_query_ctx **out);
int accx_query_ctx_free(accx_query_ctx *q);
int accx_scan_query_ctx(const accx_graph *g, accx_query_ctx *q, double eps, int mu, uint8_t *sim, int32_t *label,
                        int32_t *cluster, accx_scan_summary *summary, void *stream);

/* The sorted unique (cluster id, non-core vertex) pairs of the last query, as
 * pairs[2k] = cluster id, pairs[2k+1] = vertex; cap = capacity in pairs.  Returns
 * the count in *npairs (ACCX_ERR_TOO_LARGE when cap is short, *npairs still set). */
int accx_scan_pairs(accx_graph *g, int32_t *pairs, uint64_t cap, uint64_t *npairs, void *stream);

/* The result-file name part for eps: std::to_string(eps) with trailing '0'/'u'
 * characters removed (scan_xp_common.cu:191-192). */
int accx_eps_string(double eps, char *out, size_t cap);

/* Writes <dir>/scanxp-result-<eps>-<mu>.txt for the last query, byte-identical to
 * the reference's Graph::Output. */
int accx_write_result(accx_graph *g, const char *dir, double eps, int mu, void *stream);

/* The exact similarity predicate for one entry, on the host: cnn = cnt + 2,
 * du/dv = degree + 1.  Returns 1 when the reference's
 * (double)((long double)cnn / sqrt((long double)du*dv)) >= eps, decided in
 * exact integer arithmetic. */
int accx_similar_exact(uint32_t cnn, uint32_t du, uint32_t dv, double eps);

/* accx_similar_exact over k triples: out[i] = 0/1. */
int accx_similar_exact_batch(uint64_t k, const uint32_t *cnn, const uint32_t *du, const uint32_t *dv, double eps,
                             uint8_t *out);

/* ---- request server: continuous batching on one GPU ---------------------------
 * No reference counterpart (the reference is a single-shot CLI).  The server
 * keeps a counted graph resident and serves SCAN queries of any (eps, mu) on it,
 * plus new-graph count requests (a graph generated on the device, counted and
 * released).  Worker threads, each with its own CUDA stream and query context,
 * take requests in arrival order, first fit: a request starts as soon as a
 * worker is free and its estimated device memory fits what is left of the
 * budget, so requests arriving while others run start at once and overlap on
 * the GPU.  Every call is thread-safe. */
#define ACCX_REQ_QUERY 0
#define ACCX_REQ_COUNT 1
typedef struct {
  int type;               /* ACCX_REQ_QUERY or ACCX_REQ_COUNT */
  double eps;             /* query */
  int mu;                 /* query */
  accx_gen_params graph;  /* count: the graph to generate and count */
} accx_request;
typedef struct {
  int status;                 /* ACCX_OK or the failing call's status */
  int type;
  double queue_ms, run_ms, latency_ms;  /* submit->start, start->done, submit->done */
  accx_scan_summary summary;  /* query */
  uint64_t n, m;              /* count: the graph's size */
  uint64_t count_sum, count_digest;  /* count: accx_cn_digest of its counts */
} accx_result;
typedef struct {
  int workers;                /* concurrent requests (0 = 4) */
  uint64_t hbm_budget;        /* bytes requests may hold at once (0 = 64 GiB) */
  int count_policy;           /* policy for count requests (ACCX_POLICY_*, not TABLE) */
  int count_sm_percent;       /* SMs count requests may fill, percent (0 = 50); queries keep the rest */
  int count_orient;           /* 1: count requests relabel their graph and count oriented
                                 (accx_count_opts.orient; more HBM per request, less time) */
} accx_server_config;
typedef struct {
  uint64_t submitted, completed, failed;
  double query_p50_ms, query_p99_ms, count_p50_ms, count_p99_ms;
  double elapsed_s, throughput_rps;
  int max_concurrent;         /* most requests running at once */
  uint64_t peak_bytes;        /* most budget bytes held at once */
} accx_server_stats;
typedef struct accx_server accx_server;

/* The server reads `resident` (counted already; it is not copied) until destroyed;
 * creation waits for all work already queued on the device, so a count still
 * running on any stream is finished before the first request reads it. */
int accx_server_create(accx_graph *resident, const accx_server_config *cfg, accx_server **out);
int accx_server_submit(accx_server *s, const accx_request *req, uint64_t *id);
/* ACCX_ERR_NOT_READY while the request is pending or running. */
int accx_server_poll(accx_server *s, uint64_t id, accx_result *out);
/* Waits up to timeout_ms (< 0: no limit) for one request. */
int accx_server_wait(accx_server *s, uint64_t id, double timeout_ms, accx_result *out);
int accx_server_drain(accx_server *s);
int accx_server_stats_get(accx_server *s, accx_server_stats *out);
/* Device bytes the server would reserve for a request (its admission size). */
uint64_t accx_server_request_bytes(const accx_server *s, const accx_request *req);
int accx_server_destroy(accx_server *s);

#ifdef __cplusplus
}
#endif
#endif /* ACCX_H */

/*
 * accx_oracle.c -- CPU restatement of the reference's all-edge common-neighbour
 * count and SCAN query.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls this
 * file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it, and only as the checker (or as the timed CPU baseline), never as a
 * fallback.  Parity is pinned: tests/test_oracle_golden.py checks every function
 * here against fixtures produced by the reference's own CPU build
 * (scan-query, BIT_VEC variant) run through oracle/ref_harness.cpp.
 *
 * Reference files (paths inside the AccTriCnt tree):
 *   scan-query/util/graph.cpp:126-221       b_degree.bin / b_adj.bin loader, input checks
 *   scan-query/scan_xp.cpp:58-82            constructor: common_node_num[e] = 2, label = 0
 *   scan-query/scan_xp.cpp:220-337          CheckCoreBitmap (degree-owner rule, bitmap probe,
 *                                           symmetric assign by BinarySearch)
 *   scan-query/scan_xp.cpp:112-141          CheckCoreCompSimCore (long double predicate, cores)
 *   scan-query/scan_xp.cpp:1915-1955        ClusterCore, CheckHub, LabelNonCore
 *   scan-query/scan_xp.cpp:1983-2074        MarkClusterMinEleAsId, PrepareResultOutput
 *   scan-query/util/graph.cpp:254-294       Graph::Output (result file format)
 *   scan-query/util/union_find.h:18-35      FindRoot / Union (larger root under smaller)
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_UNCLASSIFIED 0
#define ORC_CORE 1
#define ORC_HUB 2

/* Input validation as in Graph::CheckInputGraph (graph.cpp:200-221):
 * 0 = ok, -1 = self loop, -2 = a row not strictly increasing, -3 = id out of range. */
int oracle_check_graph(uint32_t n, const uint32_t *off, const int32_t *dst) {
  for (uint32_t i = 0; i < n; i++) {
    for (uint32_t j = off[i]; j < off[i + 1]; j++) {
      if (dst[j] < 0 || (uint32_t)dst[j] >= n) return -3;
      if ((uint32_t)dst[j] == i) return -1;
      if (j > off[i] && dst[j] <= dst[j - 1]) return -2;
    }
  }
  return 0;
}

/* Recursive halving search for val inside dst[beg,end) (scan_xp.cpp:86-90); the
 * caller guarantees val is present (the graph is symmetric). */
static uint32_t orc_binary_search(const int32_t *a, uint32_t beg, uint32_t end, int32_t val) {
  for (;;) {
    uint32_t mid = (uint32_t)(((uint64_t)beg + end) / 2);
    if (a[mid] == val) return mid;
    if (val < a[mid]) end = mid; else beg = mid + 1;
    if (beg >= end) return UINT32_MAX; /* not present: asymmetric input */
  }
}

/* CheckCoreBitmap (scan_xp.cpp:220-337) with the original vertex order.
 * cnn[e] = 2 + |N(u) ∩ N(v)| for every CSR entry.  The endpoint with the larger
 * degree (ties: smaller id) owns the edge, probes the other endpoint's list
 * against a bitmap of its own list, and mirrors the value to the reverse entry.
 * Each owned edge is independent, so any thread count gives the same array.
 * Returns 0, or -4 when the graph is not symmetric. */
int oracle_cn_count(uint32_t n, const uint32_t *off, const int32_t *dst, int32_t *cnn, int nthreads) {
  uint64_t m = off[n];
  int bad = 0;
  for (uint64_t e = 0; e < m; e++) cnn[e] = 2;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : bad)
#endif
  {
    uint8_t *bits = (uint8_t *)calloc(n ? n : 1, 1);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int64_t ui = 0; ui < (int64_t)n; ui++) {
      uint32_t u = (uint32_t)ui;
      uint32_t du = off[u + 1] - off[u];
      int any_owned = 0;
      for (uint32_t e = off[u]; e < off[u + 1]; e++) {
        uint32_t v = (uint32_t)dst[e];
        uint32_t dv = off[v + 1] - off[v];
        if (du > dv || (du == dv && u < v)) { any_owned = 1; break; }
      }
      if (!any_owned) continue;
      for (uint32_t e = off[u]; e < off[u + 1]; e++) bits[dst[e]] = 1;
      for (uint32_t e = off[u]; e < off[u + 1]; e++) {
        uint32_t v = (uint32_t)dst[e];
        uint32_t dv = off[v + 1] - off[v];
        if (!(du > dv || (du == dv && u < v))) continue;
        int32_t c = 0;
        for (uint32_t f = off[v]; f < off[v + 1]; f++) c += bits[dst[f]];
        cnn[e] += c;
        uint32_t r = orc_binary_search(dst, off[v], off[v + 1], (int32_t)u);
        if (r == UINT32_MAX) { bad = 1; continue; }
        cnn[r] = cnn[e];
      }
      for (uint32_t e = off[u]; e < off[u + 1]; e++) bits[dst[e]] = 0;
    }
    free(bits);
  }
  return bad ? -4 : 0;
}

/* CheckCoreCompSimCore (scan_xp.cpp:112-141): the similarity of entry e=(u,v) is
 * (double)((long double)cnn[e] / sqrtl((long double)(d_u+1) * (d_v+1))) >= eps,
 * computed in the host's long double exactly as the reference does.  core_count
 * is accumulated per row (sequentially equal to the single-thread reference). */
void oracle_similarity(uint32_t n, const uint32_t *off, const int32_t *dst, const int32_t *cnn, double eps,
                       int mu, uint8_t *sim, int32_t *core_count, int32_t *label, int nthreads) {
  /* rows are independent (each row's core count is summed in entry order), so
   * any thread count gives the single-thread result */
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1024)
#endif
  for (int64_t ui = 0; ui < (int64_t)n; ui++) {
    const uint32_t u = (uint32_t)ui;
    int32_t cc = 0;
    for (uint32_t e = off[u]; e < off[u + 1]; e++) {
      uint32_t v = (uint32_t)dst[e];
      long double du = off[u + 1] - off[u] + 1;
      long double dv = off[v + 1] - off[v] + 1;
      double sim_value = (double)((long double)cnn[e] / sqrtl(du * dv));
      if (sim_value >= eps) { cc++; sim[e] = 1; } else { sim[e] = 0; }
    }
    core_count[u] = cc;
    label[u] = (cc >= mu) ? ORC_CORE : ORC_UNCLASSIFIED;
  }
}

/* union_find.h:18-35, sequential: FindRoot with path compression; Union links the
 * larger root under the smaller one, so a component's root is its minimum id. */
static int32_t orc_find(int32_t *parent, int32_t x) {
  int32_t r = x;
  while (parent[r] != r) r = parent[r];
  while (parent[x] != r) { int32_t nx = parent[x]; parent[x] = r; x = nx; }
  return r;
}
static void orc_union(int32_t *parent, int32_t a, int32_t b) {
  int32_t ra = orc_find(parent, a), rb = orc_find(parent, b);
  if (ra == rb) return;
  if (ra < rb) parent[rb] = ra; else parent[ra] = rb;
}

/* ClusterCore + LabelNonCore (scan_xp.cpp:1915-1955) and MarkClusterMinEleAsId
 * (scan_xp.cpp:1983-2020) for the original order.  On return label[] holds
 * 0/1/2 (UNCLASSIFIED/CORE/HUB) and cluster[u] holds the minimum vertex id of
 * u's cluster for cores, -1 for non-cores. */
void oracle_cluster(uint32_t n, const uint32_t *off, const int32_t *dst, const uint8_t *sim, int32_t *label,
                    int32_t *cluster) {
  int32_t *parent = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
  for (uint32_t i = 0; i < n; i++) parent[i] = (int32_t)i;
  for (uint32_t u = 0; u < n; u++) {
    if (label[u] != ORC_CORE) continue;
    for (uint32_t e = off[u]; e < off[u + 1]; e++) {
      int32_t v = dst[e];
      if (label[v] == ORC_CORE && sim[e]) orc_union(parent, (int32_t)u, v);
    }
  }
  for (uint32_t u = 0; u < n; u++) {
    if (label[u] == ORC_CORE) continue;
    /* CheckHub: >= 2 distinct roots among core neighbours, similarity ignored. */
    int32_t first = -1, hub = 0;
    for (uint32_t e = off[u]; e < off[u + 1] && !hub; e++) {
      int32_t v = dst[e];
      if (label[v] != ORC_CORE) continue;
      int32_t r = orc_find(parent, v);
      if (first < 0) first = r; else if (r != first) hub = 1;
    }
    if (hub) label[u] = ORC_HUB;
  }
  /* The root of every component is its minimum id, which is also the cluster id
   * MarkClusterMinEleAsId computes. */
  for (uint32_t u = 0; u < n; u++) cluster[u] = (label[u] == ORC_CORE) ? orc_find(parent, (int32_t)u) : -1;
  free(parent);
}

static int orc_pair_cmp(const void *a, const void *b) {
  const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}

/* PrepareResultOutput (scan_xp.cpp:2022-2074): the unique (cluster id, v) pairs of
 * a core u, a non-core v and a similar entry (u,v), sorted by (cluster id, v).
 * pairs[2k] = cluster id, pairs[2k+1] = v.  Returns the pair count; with
 * pairs == NULL only counts candidate entries (an upper bound). */
int64_t oracle_noncore_pairs(uint32_t n, const uint32_t *off, const int32_t *dst, const uint8_t *sim,
                             const int32_t *label, const int32_t *cluster, int32_t *pairs) {
  int64_t k = 0;
  for (uint32_t u = 0; u < n; u++) {
    if (label[u] != ORC_CORE) continue;
    for (uint32_t e = off[u]; e < off[u + 1]; e++) {
      int32_t v = dst[e];
      if (label[v] != ORC_CORE && sim[e]) k++;
    }
  }
  if (!pairs) return k;
  int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * (k ? k : 1));
  int64_t j = 0;
  for (uint32_t u = 0; u < n; u++) {
    if (label[u] != ORC_CORE) continue;
    for (uint32_t e = off[u]; e < off[u + 1]; e++) {
      int32_t v = dst[e];
      if (label[v] != ORC_CORE && sim[e]) keys[j++] = ((int64_t)cluster[u] << 32) | (uint32_t)v;
    }
  }
  qsort(keys, (size_t)k, sizeof(int64_t), orc_pair_cmp);
  int64_t w = 0;
  for (int64_t i = 0; i < k; i++) {
    if (i > 0 && keys[i] == keys[i - 1]) continue;
    pairs[2 * w] = (int32_t)(keys[i] >> 32);
    pairs[2 * w + 1] = (int32_t)(keys[i] & 0xffffffff);
    w++;
  }
  free(keys);
  return w;
}

/* The result-file name part for eps: std::to_string(eps) ("%f") with trailing
 * '0' and 'u' characters erased (scan_xp.cpp:2062-2063). */
void oracle_eps_string(double eps, char *out, int cap) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%f", eps);
  int len = (int)strlen(buf);
  while (len > 0 && (buf[len - 1] == '0' || buf[len - 1] == 'u')) len--;
  buf[len] = 0;
  snprintf(out, (size_t)cap, "%s", buf);
}

/* Graph::Output (graph.cpp:254-294): writes <dir>/scanxp-result-<eps>-<mu>.txt.
 * Returns 0 or -5 when the file cannot be opened. */
int oracle_write_result(const char *dir, double eps, int mu, uint32_t n, const int32_t *label,
                        const int32_t *cluster, const int32_t *pairs, int64_t npairs) {
  char eps_s[512], path[4096];
  oracle_eps_string(eps, eps_s, sizeof(eps_s));
  snprintf(path, sizeof(path), "%s/scanxp-result-%s-%d.txt", dir, eps_s, mu);
  FILE *f = fopen(path, "w");
  if (!f) return -5;
  fputs("c/n vertex_id cluster_id\n", f);
  for (uint32_t i = 0; i < n; i++)
    if (label[i] == ORC_CORE) fprintf(f, "c %u %d\n", i, cluster[i]);
  for (int64_t k = 0; k < npairs; k++) fprintf(f, "n %d %d\n", pairs[2 * k + 1], pairs[2 * k]);
  fclose(f);
  return 0;
}

/* Reads b_degree.bin / b_adj.bin (graph.cpp:126-198).  *n_out and *m_out receive
 * the header sizes; with off/dst NULL only the header is read.  The degree file is
 * int32 int_size, uint32 n, uint32 m, int32 degree[n]; the adjacency file is
 * int32 dst[m].  Returns 0, -6 (cannot open) or -7 (short file). */
int oracle_read_graph(const char *dir, uint32_t *n_out, uint32_t *m_out, uint32_t *off, int32_t *dst) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/b_degree.bin", dir);
  FILE *f = fopen(path, "rb");
  if (!f) return -6;
  int32_t int_size;
  uint32_t n, m;
  if (fread(&int_size, 4, 1, f) != 1 || fread(&n, 4, 1, f) != 1 || fread(&m, 4, 1, f) != 1) { fclose(f); return -7; }
  *n_out = n; *m_out = m;
  if (!off) { fclose(f); return 0; }
  off[0] = 0;
  for (uint32_t i = 0; i < n; i++) {
    int32_t d;
    if (fread(&d, 4, 1, f) != 1) { fclose(f); return -7; }
    off[i + 1] = off[i] + (uint32_t)d;
  }
  fclose(f);
  snprintf(path, sizeof(path), "%s/b_adj.bin", dir);
  f = fopen(path, "rb");
  if (!f) return -6;
  size_t got = fread(dst, 4, m, f);
  fclose(f);
  return got == m ? 0 : -7;
}

/* The whole reference pipeline on one graph: count, similarity, cores, clusters,
 * hubs, pairs and (when dir != NULL) the result file.  sim/label/cluster are
 * caller buffers of m/n/n entries; returns the number of non-core pairs or a
 * negative status. */
int64_t oracle_scan(uint32_t n, const uint32_t *off, const int32_t *dst, double eps, int mu, int nthreads,
                    int32_t *cnn, uint8_t *sim, int32_t *core_count, int32_t *label, int32_t *cluster,
                    const char *dir) {
  int rc = oracle_cn_count(n, off, dst, cnn, nthreads);
  if (rc) return rc;
  oracle_similarity(n, off, dst, cnn, eps, mu, sim, core_count, label, nthreads);
  oracle_cluster(n, off, dst, sim, label, cluster);
  int64_t k = oracle_noncore_pairs(n, off, dst, sim, label, cluster, NULL);
  int32_t *pairs = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)(k ? k : 1));
  int64_t np = oracle_noncore_pairs(n, off, dst, sim, label, cluster, pairs);
  if (dir) rc = oracle_write_result(dir, eps, mu, n, label, cluster, pairs, np);
  free(pairs);
  return rc ? rc : np;
}

/* The reference's similarity expression for one (cnn, du, dv) triple, evaluated
 * in this host's long double exactly as CheckCoreCompSimCore does; fills
 * out[i] for k triples (used to check the exact-integer predicate). */
void oracle_sim_batch(int64_t k, const uint32_t *cnn, const uint32_t *du, const uint32_t *dv, double eps,
                      uint8_t *out) {
  for (int64_t i = 0; i < k; i++) {
    long double a = du[i], b = dv[i];
    double sim_value = (double)((long double)cnn[i] / sqrtl(a * b));
    out[i] = sim_value >= eps;
  }
}

/* Row of CSR entry i, searched forward from row u (off[u] <= i): galloping, then
 * a binary search, as FindSrc does (scan_xp.cpp:94-110); returns the last row r
 * with off[r] <= i, which skips empty rows. */
static uint32_t orc_find_src(const uint32_t *off, uint32_t n, uint32_t u, uint64_t i) {
  if (i < off[u + 1]) return u;
  uint32_t lo = u + 1, step = 1, hi = lo;
  while (hi < n && off[hi + 1] <= i) { lo = hi + 1; hi = lo + step; step <<= 1; if (hi > n) hi = n; }
  if (hi > n) hi = n;
  /* first r in [lo, hi] with off[r + 1] > i */
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if (off[mid + 1] <= i) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* CheckCoreBitmap (scan_xp.cpp:219-337, the BIT_VEC build) over a stripe of its
 * entry chunks: the reference walks the CSR entries in chunks of `chunk` (6000,
 * OpenMP schedule(dynamic, 6000)); every thread keeps a bit vector of the
 * neighbours of its current row u, rebuilt (old bits cleared) when the row
 * changes; for an entry e = (u,v) that u owns (larger degree, ties: smaller id)
 * it counts the set bits over N(v), adds the count to cnn[e] (which starts at
 * 2) and copies cnn[e] to the reverse entry, found by binary search in N(v).
 * This call processes the chunks c with c % nstripes == stripe, dynamically over
 * nthreads threads, so nstripes calls (stripe 0..nstripes-1) are one whole
 * count and each is a bounded, evenly spread part of it (the timed CPU
 * baseline).  Returns the CSR entries in the stripe's chunks, -4 on an
 * asymmetric graph. */
int64_t oracle_cn_count_bitvec_stripe(uint32_t n, const uint32_t *off, const int32_t *dst, int32_t *cnn,
                                      uint32_t chunk, uint32_t stripe, uint32_t nstripes, int nthreads) {
  const uint64_t m = off[n];
  if (chunk == 0 || nstripes == 0 || stripe >= nstripes) return -1;
  const int64_t nchunks = (int64_t)((m + chunk - 1) / chunk);
  const int64_t mine = nchunks > (int64_t)stripe ? (nchunks - (int64_t)stripe + nstripes - 1) / nstripes : 0;
  const size_t words = ((size_t)n + 63) / 64;
  int64_t entries = 0;
  int bad = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(+ : entries) reduction(| : bad)
#endif
  {
    uint64_t *bits = (uint64_t *)calloc(words ? words : 1, sizeof(uint64_t));
    uint32_t u = 0;
    int64_t last_u = -1;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int64_t k = 0; k < mine; k++) {
      const uint64_t c = (uint64_t)stripe + (uint64_t)k * nstripes;
      const uint64_t e0 = c * chunk, e1 = e0 + chunk < m ? e0 + chunk : m;
      entries += (int64_t)(e1 - e0);
      if (off[u] > e0) u = 0; /* a chunk behind this thread's row: search from the start */
      for (uint64_t i = e0; i < e1; i++) {
        u = orc_find_src(off, n, u, i);
        if ((int64_t)u != last_u) {
          if (last_u >= 0)
            for (uint32_t f = off[last_u]; f < off[last_u + 1]; f++) bits[(uint32_t)dst[f] >> 6] = 0;
          for (uint32_t f = off[u]; f < off[u + 1]; f++) bits[(uint32_t)dst[f] >> 6] |= 1ull << ((uint32_t)dst[f] & 63);
          last_u = u;
        }
        const uint32_t v = (uint32_t)dst[i];
        const uint32_t du = off[u + 1] - off[u], dv = off[v + 1] - off[v];
        if (du > dv || (du == dv && u < v)) {
          int32_t cn = 0;
          for (uint32_t f = off[v]; f < off[v + 1]; f++) cn += (int32_t)((bits[(uint32_t)dst[f] >> 6] >> ((uint32_t)dst[f] & 63)) & 1u);
          cnn[i] += cn;
          const uint32_t r = orc_binary_search(dst, off[v], off[v + 1], (int32_t)u);
          if (r == UINT32_MAX) bad = 1; else cnn[r] = cnn[i];
        }
      }
    }
    free(bits);
  }
  return bad ? -4 : entries;
}

static int orc_int_cmp(const void *a, const void *b) {
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

/* The reference's "deg" reorder, ReorderDegDescending + Reorder
 * (scan_xp.cpp:1279-1301, :1145-1222): vertices sorted by degree, descending
 * (old_vid[new] = old id; the reference's parallel sort leaves equal degrees in
 * any order, this one keeps them by id), new_off from the new degrees, every
 * row's ids mapped through new_vid and sorted.  Output arrays are caller-owned:
 * new_off[n+1], new_dst[m], old_vid[n]. */
void oracle_reorder_deg(uint32_t n, const uint32_t *off, const int32_t *dst, int nthreads, uint32_t *new_off,
                        int32_t *new_dst, uint32_t *old_vid) {
  uint32_t maxd = 0;
  for (uint32_t u = 0; u < n; u++) if (off[u + 1] - off[u] > maxd) maxd = off[u + 1] - off[u];
  /* counting sort by degree, descending, stable in the id */
  uint64_t *start = (uint64_t *)calloc((size_t)maxd + 2, sizeof(uint64_t));
  for (uint32_t u = 0; u < n; u++) start[maxd - (off[u + 1] - off[u]) + 1]++;
  for (uint32_t d = 1; d <= maxd + 1; d++) start[d] += start[d - 1];
  for (uint32_t u = 0; u < n; u++) old_vid[start[maxd - (off[u + 1] - off[u])]++] = u;
  free(start);
  uint32_t *new_vid = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
  for (uint32_t i = 0; i < n; i++) new_vid[old_vid[i]] = i;
  new_off[0] = 0;
  for (uint32_t i = 0; i < n; i++) new_off[i + 1] = new_off[i] + (off[old_vid[i] + 1] - off[old_vid[i]]);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 100)
#endif
  for (int64_t ii = 0; ii < (int64_t)n; ii++) {
    const uint32_t i = (uint32_t)ii, o = old_vid[i];
    uint32_t k = new_off[i];
    for (uint32_t f = off[o]; f < off[o + 1]; f++) new_dst[k++] = (int32_t)new_vid[(uint32_t)dst[f]];
    const uint32_t len = new_off[i + 1] - new_off[i];
    if (len > 1) qsort(new_dst + new_off[i], len, sizeof(int32_t), orc_int_cmp);
  }
  free(new_vid);
}

/* ComputeVertexRangeAccumulatedFilteredDegree
 * (scan-query-cuda/scan_xp_multi_gpu_multi_pass_common.cu:516-554): cost(u) =
 * sum over v in N(u), v >= u (lower_bound of u in N(u)) of (deg v + 2); the
 * exclusive prefix over vertices is cut at total/parts*i by lower_bound.  The
 * per-vertex cost is kept in 64 bits (the reference's uint32 can wrap for hubs). */
void oracle_vertex_ranges(uint32_t n, const uint32_t *off, const int32_t *dst, int parts, uint32_t *ranges) {
  uint64_t *prefix = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)n + 1));
  prefix[0] = 0;
  for (uint32_t u = 0; u < n; u++) {
    uint64_t c = 0;
    for (uint32_t j = off[u]; j < off[u + 1]; j++) {
      uint32_t v = (uint32_t)dst[j];
      if (v >= u) c += off[v + 1] - off[v] + 2;
    }
    prefix[u + 1] = prefix[u] + c;
  }
  ranges[0] = 0;
  for (int i = 1; i < parts; i++) {
    uint64_t target = prefix[n] / (uint64_t)parts * (uint64_t)i;
    uint32_t lo = 0, hi = n + 1; /* first index with prefix >= target */
    while (lo < hi) {
      uint32_t mid = lo + (hi - lo) / 2;
      if (prefix[mid] < target) lo = mid + 1; else hi = mid;
    }
    ranges[i] = lo;
  }
  ranges[parts] = n;
  free(prefix);
}

// Learned kernel scheduler: training data, training, whole-count calibration,
// the count plan and the model file -- the host side of the cost model, behind
// the C ABI so that the C++ drop-in (SCAN_XP) and any binding use the same code.
//
// The reference has no counterpart: its kernel choice is fixed at link time
// (each CMake target compiles its own SCAN_XP::CheckCore,
// scan-query-cuda/CMakeLists.txt:114-117) and, inside the hybrid build, by a
// degree ratio of 50 (scan_xp_multi_gpu_multi_pass_common.cu:57-59, :105-117).
// Here:
//   * training data are timings the counting kernels themselves produce: for
//     every populated degree bucket and every kernel kind one count runs with
//     only that bucket enabled (the others ACCX_KIND_SKIP), timed by the
//     library's CUDA events (accx_bucket_timings);
//   * each of the two models (direct and oriented kernels) is trained with the
//     library's own FP16/FP32 training kernels on the rows of seven seeded
//     graphs -- three candidates from different seeds on the same rows, since
//     the per-bucket timings are noisy and a fit can extrapolate badly to large
//     buckets -- then calibrated on whole counts: per-bucket timings taken alone
//     overstate the bitmap kind (its owner staging serves all of an owner's
//     buckets), so the candidate and one log2 offset for that kind (among ten)
//     are chosen by the size-weighted count time on the calibration graphs;
//   * a plan attaches both models to a graph, predicts each mode's time from
//     its own table and picks the faster mode; optionally it refines the
//     chosen mode's offset on the graph itself by timing one whole count per
//     candidate.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <string>
#include <vector>

#include "accx_internal.h"

#define NB ACCX_NB
#define NBK (ACCX_NB * ACCX_NB)

// Bitmap-kind log2 offsets: negative ones favour the bitmap kind (-64: every
// bucket), positive ones the merge and galloping kinds (64: no bucket; on the
// Erdos-Renyi graph, where owners have short prefixes, galloping everywhere is the
// fastest fixed policy).
static const float kOffsets[ACCX_SCHED_NOFFSETS] = {0.0f, -0.5f, -1.0f, -1.5f, -2.0f,
                                                    -3.0f, -5.0f, -64.0f, 1.0f, 64.0f};

struct accx_sched {
  accx_model *model[2] = {nullptr, nullptr};
  accx_sched_info info{};
};

using clk = std::chrono::steady_clock;
static double secs_since(clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); }

static accx_gen_params rmat(uint64_t scale, uint64_t ef, uint64_t seed) {
  accx_gen_params p{};
  p.kind = ACCX_GEN_RMAT;
  p.p0 = scale;
  p.p1 = ef;
  p.q0 = 0.57;
  p.q1 = 0.19;
  p.q2 = 0.19;
  p.seed = seed;
  return p;
}
static accx_gen_params er(uint64_t n, uint64_t mean, uint64_t seed) {
  accx_gen_params p{};
  p.kind = ACCX_GEN_ER;
  p.p0 = n;
  p.p1 = n * mean / 2;
  p.seed = seed;
  return p;
}
static accx_gen_params chung_lu(uint64_t n, uint64_t mean, double gamma, double maxdeg, uint64_t seed) {
  accx_gen_params p{};
  p.kind = ACCX_GEN_CHUNG_LU;
  p.p0 = n;
  p.p1 = n * mean / 2;
  p.q0 = gamma;
  p.q1 = maxdeg;
  p.seed = seed;
  return p;
}

// Training graphs: R-MAT at four sizes and two edge factors, Erdos-Renyi, and
// two power laws; calibration adds R-MAT 20 and 22 so that large graphs decide.
static std::vector<accx_gen_params> training_graphs(int quick) {
  if (quick)
    return {rmat(12, 16, 11), rmat(13, 8, 12), er(1 << 13, 16, 15), chung_lu(1 << 14, 12, 2.1, 2000, 16)};
  return {rmat(16, 16, 11), rmat(17, 16, 12), rmat(18, 16, 13), rmat(19, 8, 14), er(1 << 17, 24, 15),
          chung_lu(1 << 18, 24, 2.1, 20000, 16), chung_lu(1 << 17, 12, 2.5, 5000, 17)};
}
static std::vector<accx_gen_params> calibration_graphs(int quick) {
  std::vector<accx_gen_params> g = training_graphs(quick);
  if (!quick) {
    g.push_back(rmat(20, 16, 18));
    g.push_back(rmat(22, 16, 19));
  }
  return g;
}

// Counting-phase time (merge + gallop + bitmap, ms; with `whole`, every phase of
// the count) of one count with `table`, best of reps.
static int table_count_ms(accx_graph *g, const uint8_t *table, int orient, int reps, cudaStream_t s, double *ms,
                          bool whole = false) {
  accx_count_opts o;
  memset(&o, 0, sizeof(o));
  o.policy = ACCX_POLICY_TABLE;
  o.table = table;
  o.timing = 1;
  o.orient = orient;
  double best = -1;
  for (int r = 0; r < reps; r++) {
    int rc = accx_cn_count(g, &o, nullptr, s);
    if (rc) return rc;
    float ph[ACCX_NUM_PHASES];
    rc = accx_cn_last_timings(g, ph);
    if (rc) return rc;
    double t = (double)ph[ACCX_PHASE_MERGE] + ph[ACCX_PHASE_GALLOP] + ph[ACCX_PHASE_BITMAP];
    if (whole) t += (double)ph[ACCX_PHASE_PLAN] + ph[ACCX_PHASE_MIRROR];
    if (best < 0 || t < best) best = t;
  }
  *ms = best;
  return ACCX_OK;
}

extern "C" int accx_bucket_timings(accx_graph *g, int orient, int reps, uint64_t min_edges, uint64_t *edges,
                                   float *ms, void *stream) {
  if (!g || !edges || !ms || reps < 1 || (orient != 0 && orient != 1)) return ACCX_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<double> so(NBK), sp(NBK);
  int rc = orient ? accx_bucket_stats_oriented(g, edges, so.data(), sp.data())
                  : accx_bucket_stats(g, edges, so.data(), sp.data());
  if (rc) return rc;
  for (int i = 0; i < NBK * ACCX_NUM_KINDS; i++) ms[i] = NAN;
  uint8_t t[NBK];
  memset(t, ACCX_KIND_SKIP, sizeof(t));
  double base = 0, x = 0;
  rc = table_count_ms(g, t, orient, 1, s, &x);  // warm
  if (!rc) rc = table_count_ms(g, t, orient, reps > 3 ? reps : 3, s, &base);
  if (rc) return rc;
  if (min_edges < 1) min_edges = 1;
  for (int b = 0; b < NBK; b++) {
    if (edges[b] < min_edges) continue;
    for (int k = 0; k < ACCX_NUM_KINDS; k++) {
      t[b] = (uint8_t)k;
      rc = table_count_ms(g, t, orient, reps, s, &x);
      if (rc) return rc;
      ms[b * ACCX_NUM_KINDS + k] = (float)fmax(x - base, 1e-4);
    }
    t[b] = ACCX_KIND_SKIP;
  }
  return ACCX_OK;
}

struct rows {
  std::vector<float> x, y;
  std::vector<int32_t> k;
};

// Training rows of one graph: (bucket features, kind, log2 seconds per edge) for
// buckets with at least 32 owned edges.
static int collect_graph(const accx_gen_params &p, int orient, int reps, rows *out) {
  accx_graph *g = nullptr;
  int rc = accx_graph_generate(&p, nullptr, &g);
  if (rc) return rc;
  std::vector<uint64_t> e(NBK);
  std::vector<float> T(NBK * ACCX_NUM_KINDS), X(NBK * ACCX_MODEL_IN);
  rc = accx_graph_relabel(g, nullptr);
  if (!rc) rc = accx_bucket_timings(g, orient, reps, 1, e.data(), T.data(), nullptr);
  if (!rc) rc = orient ? accx_bucket_features_oriented(g, X.data()) : accx_bucket_features(g, X.data());
  accx_graph_free(g);
  if (rc) return rc;
  for (int b = 0; b < NBK; b++) {
    if (e[b] < 32) continue;
    for (int k = 0; k < ACCX_NUM_KINDS; k++) {
      const float t = T[b * ACCX_NUM_KINDS + k];
      if (!isfinite(t)) continue;
      out->x.insert(out->x.end(), X.begin() + (size_t)b * ACCX_MODEL_IN, X.begin() + (size_t)(b + 1) * ACCX_MODEL_IN);
      out->k.push_back(k);
      out->y.push_back((float)log2((double)t * 1e-3 / (double)e[b]));
    }
  }
  return ACCX_OK;
}

static int set_offset(accx_model *m, float off) {
  const float b[ACCX_MODEL_OUT] = {0.f, 0.f, off};
  return accx_model_set_kind_bias(m, b);
}

static int model_table(accx_model *m, accx_graph *g, int orient, uint8_t *t) {
  return orient ? accx_model_table_for_oriented(m, g, t) : accx_model_table_for(m, g, t);
}

// The candidate model and the bitmap kind's offset fitted on whole counts (see
// the file comment): every candidate's table at every offset is timed on each
// calibration graph; score = sum over graphs of weight x time / that graph's
// best time over all candidates and offsets, weight = the graph's share of the
// calibration set's CSR entries.  The lowest score wins; ties keep the earlier
// candidate and the smaller offset.  relative[] gets the winner's scores.
static int calibrate(accx_model *const *ms, int K, int orient, int quick, int *chosen_model, float *chosen,
                     float *relative, float *cand_score) {
  const std::vector<accx_gen_params> gs = calibration_graphs(quick);
  const size_t G = gs.size(), NO = ACCX_SCHED_NOFFSETS;
  std::vector<double> t((size_t)K * G * NO), w(G);
  for (size_t gi = 0; gi < G; gi++) {
    accx_graph *g = nullptr;
    int rc = accx_graph_generate(&gs[gi], nullptr, &g);
    if (rc) return rc;
    rc = accx_graph_relabel(g, nullptr);
    uint32_t n = 0;
    uint64_t mm = 0;
    accx_graph_size(g, &n, &mm);
    w[gi] = (double)mm;
    for (int k = 0; k < K && !rc; k++)
      for (size_t c = 0; c < NO && !rc; c++) {
        uint8_t tab[NBK];
        rc = set_offset(ms[k], kOffsets[c]);
        if (!rc) rc = model_table(ms[k], g, orient, tab);
        if (!rc) rc = table_count_ms(g, tab, orient, quick ? 2 : 3, nullptr, &t[((size_t)k * G + gi) * NO + c]);
      }
    accx_graph_free(g);
    if (rc) return rc;
  }
  double wsum = 0;
  for (double x : w) wsum += x;
  std::vector<double> mn(G);
  for (size_t gi = 0; gi < G; gi++) {
    mn[gi] = t[gi * NO];
    for (int k = 0; k < K; k++)
      for (size_t c = 0; c < NO; c++) mn[gi] = fmin(mn[gi], t[((size_t)k * G + gi) * NO + c]);
  }
  auto score = [&](int k, size_t c) {
    double sc = 0;
    for (size_t gi = 0; gi < G; gi++)
      sc += (wsum > 0 ? w[gi] / wsum : 0.0) * (mn[gi] > 0 ? t[((size_t)k * G + gi) * NO + c] / mn[gi] : 1.0);
    return sc;
  };
  double best = 0;
  int bk = 0;
  size_t bc = 0;
  for (int k = 0; k < K; k++) {
    double kb = 0;
    for (size_t c = 0; c < NO; c++) {
      const double sc = score(k, c);
      if (c == 0 || sc < kb) kb = sc;
      if ((k == 0 && c == 0) || sc < best) {
        best = sc;
        bk = k;
        bc = c;
      }
    }
    cand_score[k] = (float)kb;
  }
  for (size_t c = 0; c < NO; c++) relative[c] = (float)score(bk, c);
  *chosen_model = bk;
  *chosen = kOffsets[bc];
  return set_offset(ms[bk], kOffsets[bc]);
}

// Training of one mode's model: rows collected once, K candidates trained on
// them from different seeds, the calibration keeps one.
static int train_one(accx_sched *s, int orient, const accx_sched_config &c) {
  auto t0 = clk::now();
  rows r;
  for (const accx_gen_params &p : training_graphs(c.quick)) {
    int rc = collect_graph(p, orient, c.reps, &r);
    if (rc) return rc;
  }
  if (r.k.empty()) return ACCX_ERR_NOT_READY;
  s->info.collect_s[orient] = secs_since(t0);
  s->info.rows[orient] = (uint32_t)r.k.size();
  const int K = c.candidates;
  std::vector<accx_model *> ms(K, nullptr);
  std::vector<float> l0(K), l1(K);
  int rc = ACCX_OK;
  t0 = clk::now();
  for (int k = 0; k < K && !rc; k++) {
    rc = accx_model_create(c.seed + (uint64_t)k, &ms[k]);
    if (!rc) rc = accx_model_loss_grad(ms[k], r.x.data(), r.k.data(), r.y.data(), (uint32_t)r.k.size(), nullptr, &l0[k]);
    if (!rc) rc = accx_model_train(ms[k], r.x.data(), r.k.data(), r.y.data(), (uint32_t)r.k.size(), c.epochs, c.lr, &l1[k]);
  }
  s->info.train_s[orient] = secs_since(t0);
  int ck = 0;
  if (!rc) {
    t0 = clk::now();
    rc = calibrate(ms.data(), K, orient, c.quick, &ck, &s->info.bitmap_offset[orient], s->info.calib_relative[orient],
                   s->info.candidate_score[orient]);
    s->info.calibrate_s[orient] = secs_since(t0);
  }
  for (int k = 0; k < K; k++)
    if (ms[k] && (rc || k != ck)) accx_model_free(ms[k]);
  if (rc) return rc;
  s->model[orient] = ms[ck];
  s->info.candidates[orient] = K;
  s->info.chosen[orient] = ck;
  s->info.loss_initial[orient] = l0[ck];
  s->info.loss_final[orient] = l1[ck];
  return ACCX_OK;
}

extern "C" int accx_sched_train(const accx_sched_config *cfg, accx_sched **out) {
  if (!out) return ACCX_ERR_INVALID_ARG;
  accx_sched_config c;
  memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if (!c.seed) c.seed = 1;
  if (c.epochs <= 0) c.epochs = c.quick ? 800 : 4000;
  if (!(c.lr > 0)) c.lr = 3e-3f;
  if (c.reps <= 0) c.reps = 2;
  if (c.candidates <= 0) c.candidates = c.quick ? 1 : 3;
  if (c.candidates > ACCX_SCHED_MAX_CANDIDATES) return ACCX_ERR_INVALID_ARG;
  accx_sched *s = new (std::nothrow) accx_sched();
  if (!s) return ACCX_ERR_OOM;
  s->info.quick = c.quick;
  for (int orient = 0; orient < 2; orient++) {
    int rc = train_one(s, orient, c);
    if (rc) {
      accx_sched_free(s);
      return rc;
    }
  }
  *out = s;
  return ACCX_OK;
}

extern "C" int accx_sched_free(accx_sched *s) {
  if (!s) return ACCX_ERR_INVALID_ARG;
  for (accx_model *m : s->model)
    if (m) accx_model_free(m);
  delete s;
  return ACCX_OK;
}

extern "C" int accx_sched_model(accx_sched *s, int orient, accx_model **out) {
  if (!s || !out || (orient != 0 && orient != 1) || !s->model[orient]) return ACCX_ERR_INVALID_ARG;
  *out = s->model[orient];
  return ACCX_OK;
}

extern "C" int accx_sched_get_info(const accx_sched *s, accx_sched_info *info) {
  if (!s || !info) return ACCX_ERR_INVALID_ARG;
  *info = s->info;
  return ACCX_OK;
}

// File: text, "accx-sched 2", then per model (direct, then oriented) a line
// "model <orient> <kind bias x3>", a line of ACCX_MODEL_NPARAMS parameters and an
// info line (version 2 ends it with the candidates, the one kept and
// ACCX_SCHED_MAX_CANDIDATES scores; version 1 files, without them, still load);
// floats in %.9g (round trip exact for FP32).
extern "C" int accx_sched_save(const accx_sched *s, const char *path) {
  if (!s || !path || !s->model[0] || !s->model[1]) return ACCX_ERR_INVALID_ARG;
  FILE *f = fopen(path, "w");
  if (!f) return ACCX_ERR_IO;
  fprintf(f, "accx-sched 2\n");
  for (int o = 0; o < 2; o++) {
    float b[ACCX_MODEL_OUT], p[ACCX_MODEL_NPARAMS];
    int rc = accx_model_get_kind_bias(s->model[o], b);
    if (!rc) rc = accx_model_get_params(s->model[o], p);
    if (rc) {
      fclose(f);
      return rc;
    }
    fprintf(f, "model %d %.9g %.9g %.9g\n", o, b[0], b[1], b[2]);
    for (int i = 0; i < ACCX_MODEL_NPARAMS; i++) fprintf(f, "%.9g%c", p[i], i + 1 < ACCX_MODEL_NPARAMS ? ' ' : '\n');
    const accx_sched_info &in = s->info;
    fprintf(f, "info %u %.9g %.9g %.9g %.6f %.6f %.6f %d", in.rows[o], in.loss_initial[o], in.loss_final[o],
            in.bitmap_offset[o], in.collect_s[o], in.train_s[o], in.calibrate_s[o], in.quick);
    for (int c = 0; c < ACCX_SCHED_NOFFSETS; c++) fprintf(f, " %.9g", in.calib_relative[o][c]);
    fprintf(f, " %d %d", in.candidates[o], in.chosen[o]);
    for (int k = 0; k < ACCX_SCHED_MAX_CANDIDATES; k++) fprintf(f, " %.9g", in.candidate_score[o][k]);
    fprintf(f, "\n");
  }
  const bool ok = !ferror(f);
  return (fclose(f) == 0 && ok) ? ACCX_OK : ACCX_ERR_IO;
}

extern "C" int accx_sched_load(const char *path, accx_sched **out) {
  if (!path || !out) return ACCX_ERR_INVALID_ARG;
  FILE *f = fopen(path, "r");
  if (!f) return ACCX_ERR_IO;
  accx_sched *s = new (std::nothrow) accx_sched();
  if (!s) {
    fclose(f);
    return ACCX_ERR_OOM;
  }
  int rc = ACCX_OK, ver = 0;
  if (fscanf(f, " accx-sched %d", &ver) != 1 || (ver != 1 && ver != 2)) rc = ACCX_ERR_IO;
  for (int o = 0; o < 2 && !rc; o++) {
    int oo = -1;
    float b[ACCX_MODEL_OUT], p[ACCX_MODEL_NPARAMS];
    if (fscanf(f, " model %d %f %f %f", &oo, &b[0], &b[1], &b[2]) != 4 || oo != o) {
      rc = ACCX_ERR_IO;
      break;
    }
    for (int i = 0; i < ACCX_MODEL_NPARAMS && !rc; i++)
      if (fscanf(f, " %f", &p[i]) != 1) rc = ACCX_ERR_IO;
    accx_sched_info &in = s->info;
    if (!rc && fscanf(f, " info %u %f %f %f %lf %lf %lf %d", &in.rows[o], &in.loss_initial[o], &in.loss_final[o],
                      &in.bitmap_offset[o], &in.collect_s[o], &in.train_s[o], &in.calibrate_s[o], &in.quick) != 8)
      rc = ACCX_ERR_IO;
    for (int c = 0; c < ACCX_SCHED_NOFFSETS && !rc; c++)
      if (fscanf(f, " %f", &in.calib_relative[o][c]) != 1) rc = ACCX_ERR_IO;
    if (!rc && ver >= 2) {  // version 2 adds the candidates record
      if (fscanf(f, " %d %d", &in.candidates[o], &in.chosen[o]) != 2) rc = ACCX_ERR_IO;
      for (int k = 0; k < ACCX_SCHED_MAX_CANDIDATES && !rc; k++)
        if (fscanf(f, " %f", &in.candidate_score[o][k]) != 1) rc = ACCX_ERR_IO;
    }
    if (!rc) rc = accx_model_create(1, &s->model[o]);
    if (!rc) rc = accx_model_set_params(s->model[o], p);
    if (!rc) rc = accx_model_set_kind_bias(s->model[o], b);
  }
  fclose(f);
  if (rc) {
    accx_sched_free(s);
    return rc;
  }
  *out = s;
  return ACCX_OK;
}

extern "C" int accx_sched_plan_for(accx_sched *s, accx_graph *g, int tune, accx_count_opts *opts,
                                   accx_sched_plan *plan, void *stream) {
  if (!s || !g || !s->model[0] || !s->model[1]) return ACCX_ERR_INVALID_ARG;
  accx_sched_plan pl;
  memset(&pl, 0, sizeof(pl));
  int rc = accx_graph_set_model(g, s->model[0]);
  if (!rc) rc = accx_graph_set_model_oriented(g, s->model[1]);
  if (!rc) rc = accx_model_plan_ms(s->model[0], g, 0, (cudaStream_t)stream, &pl.predicted_ms[0]);
  if (!rc) rc = accx_model_plan_ms(s->model[1], g, 1, (cudaStream_t)stream, &pl.predicted_ms[1]);
  if (rc) return rc;
  pl.orient = pl.predicted_ms[1] < pl.predicted_ms[0] ? 1 : 0;
  auto t0 = clk::now();
  if (tune) {
    // the mode by measurement: each mode's own table as a whole count (every
    // phase), best of two; the predictions extrapolate poorly to graphs far from
    // the training set (an Erdos-Renyi graph 150x the training one)
    for (int o = 0; o < 2; o++) {
      uint8_t t[NBK];
      double ms = 0;
      rc = model_table(s->model[o], g, o, t);
      if (!rc) rc = table_count_ms(g, t, o, 2, (cudaStream_t)stream, &ms, true);
      if (rc) return rc;
      pl.mode_ms[o] = ms;
    }
    pl.orient = pl.mode_ms[1] < pl.mode_ms[0] ? 1 : 0;
  }
  accx_model *m = s->model[pl.orient];
  float b[ACCX_MODEL_OUT];
  rc = accx_model_get_kind_bias(m, b);
  if (rc) return rc;
  pl.bitmap_offset = b[2];
  pl.calibrated_offset = b[2];
  if (tune) {
    // one whole count per candidate offset on this graph; ties keep the offset in use
    int bi = -1;
    double best = 0;
    for (int c = 0; c < ACCX_SCHED_NOFFSETS; c++) {
      uint8_t t[NBK];
      double ms = 0;
      rc = set_offset(m, kOffsets[c]);
      if (!rc) rc = model_table(m, g, pl.orient, t);
      if (!rc) rc = table_count_ms(g, t, pl.orient, 2, (cudaStream_t)stream, &ms);
      if (rc) {
        set_offset(m, pl.calibrated_offset);
        return rc;
      }
      pl.tune_ms[c] = (float)ms;
      if (bi < 0 || ms < best) {
        best = ms;
        bi = c;
      }
    }
    for (int c = 0; c < ACCX_SCHED_NOFFSETS; c++)
      if (kOffsets[c] == pl.calibrated_offset && pl.tune_ms[c] <= best) bi = c;
    pl.bitmap_offset = kOffsets[bi];
    rc = set_offset(m, pl.bitmap_offset);
    if (rc) return rc;
    pl.tuned = 1;
    pl.tune_s = secs_since(t0);
  }
  for (int c = 0; c < ACCX_SCHED_NOFFSETS; c++) pl.offsets[c] = kOffsets[c];
  if (opts) {
    memset(opts, 0, sizeof(*opts));
    opts->policy = ACCX_POLICY_MODEL;
    opts->orient = pl.orient;
  }
  if (plan) *plan = pl;
  return ACCX_OK;
}

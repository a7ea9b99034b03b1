// SCAN_XP on libaccx: the reference's Execute() sequence
// (scan-query-cuda/scan_xp_common.cu:334-360), each phase one or two C ABI calls.
#include "scan_xp.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include <chrono>
#include <stdexcept>
#include <string>

static FILE *g_log_file = nullptr;

void accx_log_set_file(const char *path) {
  if (g_log_file) fclose(g_log_file);
  g_log_file = path ? fopen(path, "a+") : nullptr;
}

void accx_log(const char *fmt, ...) {
  char msg[2048];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  time_t t = time(nullptr);
  char ts[32];
  strftime(ts, sizeof(ts), "%H:%M:%S", localtime(&t));
  printf("%s INFO %s\n", ts, msg);
  fflush(stdout);
  if (g_log_file) {
    fprintf(g_log_file, "%s INFO %s\n", ts, msg);
    fflush(g_log_file);
  }
}

static void check(int rc, const char *what) {
  if (rc != ACCX_OK) throw std::runtime_error(std::string(what) + ": " + accx_strerror(rc));
}

ScanXpOptions ScanXpOptions::from_env() {
  ScanXpOptions o;
  const char *p = getenv("ACCX_POLICY");
  if (p) {
    std::string s(p);
    if (s == "heuristic") o.policy = ACCX_POLICY_HEURISTIC;
    else if (s == "merge") o.policy = ACCX_POLICY_MERGE;
    else if (s == "gallop") o.policy = ACCX_POLICY_GALLOP;
    else if (s == "bitmap") o.policy = ACCX_POLICY_BITMAP;
    else if (s == "model") o.policy = ACCX_POLICY_MODEL;
    else o.policy = ACCX_POLICY_TABLE;
    o.policy_set = true;
  }
  const char *r = getenv("ACCX_RELABEL");
  if (r) o.relabel = atoi(r) != 0;
  const char *q = getenv("ACCX_ORIENT");
  if (q) o.orient = atoi(q) != 0;
  const char *m = getenv("ACCX_SCHED_MODEL");
  if (m) o.sched_path = m;
  const char *t = getenv("ACCX_SCHED_TUNE");
  if (t) o.sched_tune = atoi(t) != 0;
  return o;
}

// <directory of this executable>/accx-sched.model: where the build puts the
// scheduler file it trains.
static std::string default_sched_path() {
  char buf[4096];
  const ssize_t k = readlink("/proc/self/exe", buf, sizeof(buf) - 1);
  if (k <= 0) return "accx-sched.model";
  buf[k] = 0;
  std::string p(buf);
  const size_t slash = p.rfind('/');
  return (slash == std::string::npos ? std::string(".") : p.substr(0, slash)) + "/accx-sched.model";
}

// Default bucket table: galloping where the owner's degree bucket exceeds the
// other's by 6 or more (ratio >= 64), the shared-memory bitmap for owners of
// degree >= 256, warp merge below.
static void default_table(uint8_t *t) {
  for (int a = 0; a < ACCX_NB; a++)
    for (int b = 0; b < ACCX_NB; b++)
      t[a * ACCX_NB + b] = a >= 8 ? ACCX_KIND_BITMAP : (a - b >= 6 ? ACCX_KIND_GALLOP : ACCX_KIND_MERGE);
}

using clk = std::chrono::steady_clock;
static double secs(clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); }

SCAN_XP::SCAN_XP(int thread_num, int min_u, double epsilon, char *dir)
    : SCAN_XP(thread_num, min_u, epsilon, dir, ScanXpOptions::from_env()) {}

SCAN_XP::SCAN_XP(int thread_num, int min_u, double epsilon, char *dir, const ScanXpOptions &opts)
    : min_u_(min_u), epsilon_(epsilon), dir_(dir ? dir : ""), opts_(opts), thread_num_(thread_num) {
  auto t0 = clk::now();
  check(accx_graph_load_dir(dir_.c_str(), ACCX_GRAPH_VALIDATE, nullptr, &g_), "load graph");
  uint32_t n = 0;
  uint64_t m = 0;
  accx_graph_size(g_, &n, &m);
  accx_log("graph dir: %s", dir_.c_str());
  accx_log("thread num: %d", thread_num_);
  accx_log("graph, n: %u, m: %llu (loaded and checked in %.3lf s)", n, (unsigned long long)m, secs(t0));
  if (opts_.relabel) {
    t0 = clk::now();
    check(accx_graph_relabel(g_, nullptr), "relabel");
    accx_log("PreProcess Reordering Cost (GPU degree-descending): %.3lf s", secs(t0));
  }
}

SCAN_XP::~SCAN_XP() {
  if (sched_) accx_sched_free(sched_);
  if (g_) accx_graph_free(g_);
}

void SCAN_XP::CheckCore() {
  uint8_t table[ACCX_NB * ACCX_NB];
  default_table(table);
  accx_count_opts o;
  memset(&o, 0, sizeof(o));
  auto t0 = clk::now();
  if (opts_.policy_set) {
    o.policy = opts_.policy;
    o.table = table;
    o.orient = opts_.orient ? 1 : 0;
    accx_log("kernel plan: policy %d from ACCX_POLICY (%s)", o.policy, o.orient ? "oriented" : "direct");
  } else {
    const std::string path = opts_.sched_path.empty() ? default_sched_path() : opts_.sched_path;
    accx_sched_plan pl;
    if (accx_sched_load(path.c_str(), &sched_) == ACCX_OK) {
      check(accx_sched_plan_for(sched_, g_, opts_.sched_tune ? 1 : 0, &o, &pl, nullptr), "scheduler plan");
      accx_log("kernel plan: learned scheduler %s -> %s counting (predicted %.3lf ms direct, %.3lf ms oriented; "
               "bitmap offset %.2f)", path.c_str(), pl.orient ? "oriented" : "direct", pl.predicted_ms[0],
               pl.predicted_ms[1], pl.bitmap_offset);
    } else {
      // the reference's fixed rule: ratio-50 galloping, else merge, full lists
      o.policy = ACCX_POLICY_HEURISTIC;
      o.orient = 0;
      accx_log("kernel plan: reference ratio-50 rule (no scheduler file at %s)", path.c_str());
    }
  }
  o.bias = 2;  // common_node_num = 2 + |N(u) ∩ N(v)|
  o.block_warps = opts_.block_warps;
  check(accx_cn_count(g_, &o, nullptr, nullptr), "count");
  check(accx_scan_query(g_, epsilon_, min_u_, nullptr, nullptr, nullptr, &summary, nullptr), "similarity");
  accx_log("All-Edge CN-Cnt + core checking (GPU, %s): %.3lf s", o.orient ? "oriented" : "direct", secs(t0));
}

void SCAN_XP::ClusterCore() {
  // union-find, hubs and outliers ran with the query; report as the reference does
  accx_log("Core: %u", summary.cores);
}

void SCAN_XP::PostProcess() {
  accx_log("Cluster: %u, Hub: %u, Outlier: %u", summary.clusters, summary.hubs, summary.outliers);
}

void SCAN_XP::PrepareResultOutput() {
  auto t0 = clk::now();
  check(accx_write_result(g_, dir_.c_str(), epsilon_, min_u_, nullptr), "write result");
  accx_log("Step4 - output to the disk cost: %.3lf s", secs(t0));
}

void SCAN_XP::Execute() {
  auto t0 = clk::now();
  CheckCore();
  accx_log("Step1 - CheckCore: %.3lf s", secs(t0));
  t0 = clk::now();
  ClusterCore();
  accx_log("Step2 - ClusterCore: %.3lf s", secs(t0));
  PostProcess();
  PrepareResultOutput();
}

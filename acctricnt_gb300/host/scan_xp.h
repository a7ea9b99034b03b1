// SCAN_XP: the reference's SCAN query class, on libaccx.
//
// Same public surface as the reference (scan-query-cuda/scan_xp.h:21-59):
// SCAN_XP(int thread_num, int min_u, double epsilon, char *dir) loads
// <dir>/b_degree.bin and <dir>/b_adj.bin, and Execute() runs the all-edge count
// (CheckCore), core detection, clustering, hub/outlier labelling and writes
// <dir>/scanxp-result-<eps>-<mu>.txt byte-identical to the reference.  All work
// runs on the GPU through the C ABI (include/accx.h); errors surface as
// std::runtime_error instead of exit().
#ifndef ACCX_SCAN_XP_H
#define ACCX_SCAN_XP_H

#include <string>

#include "accx.h"

// How CheckCore picks its kernels.  Without an explicit policy it loads the
// learned scheduler's file (accx_sched_load) and counts with the plan the
// scheduler makes for the graph (mode and per-bucket kinds from the cost
// models); when there is no usable file it falls back to the reference's own
// rule, galloping iff one degree exceeds 50x the other, else merging, over full
// lists (scan_xp_multi_gpu_multi_pass_common.cu:57-59, :105-117).  The counts
// are the same either way.
struct ScanXpOptions {
  int policy = ACCX_POLICY_TABLE;  // explicit counting policy (ACCX_POLICY_*); TABLE uses the default bucket table
  bool policy_set = false;         // a policy chosen by the caller (else: scheduler, or the ratio-50 fallback)
  bool relabel = true;             // count on the degree-descending relabeled copy
  bool orient = true;              // with an explicit policy: oriented counting (same counts)
  int block_warps = 0;             // bitmap/merge CTA size in warps (0 = default)
  std::string sched_path;          // scheduler file ("" = <directory of the executable>/accx-sched.model)
  bool sched_tune = false;         // refine the bitmap offset on this graph (a whole count per candidate)
  // ACCX_POLICY=heuristic|merge|gallop|bitmap|table|model, ACCX_RELABEL=0|1, ACCX_ORIENT=0|1,
  // ACCX_SCHED_MODEL=<file>, ACCX_SCHED_TUNE=0|1
  static ScanXpOptions from_env();
};

class SCAN_XP {
 private:
  int min_u_;
  double epsilon_;
  std::string dir_;
  accx_graph *g_ = nullptr;
  accx_sched *sched_ = nullptr;
  ScanXpOptions opts_;

  void CheckCore();   // all-edge counts (+2 closed-neighbourhood bias) and cores
  void ClusterCore(); // union-find over similar core-core edges, hubs, outliers
  void PostProcess();
  void PrepareResultOutput();

 public:
  int thread_num_;

  SCAN_XP(int thread_num, int min_u, double epsilon, char *dir);
  SCAN_XP(int thread_num, int min_u, double epsilon, char *dir, const ScanXpOptions &opts);
  ~SCAN_XP();

  void Execute();

  accx_scan_summary summary{};  // cores, clusters, hubs, outliers of the last Execute
};

// Log sink shared by the CLIs: lines "<time> INFO <message>" to stdout and, when
// set, appended to a file (the reference's log_set_fp(fopen(path, "a+"))).
void accx_log_set_file(const char *path);
void accx_log(const char *fmt, ...);

#endif

// CLI of the reference's scan-query-cuda/experimental/main_scanxp.cpp:17-44:
//   scan-xp-gb300-varying <graph-dir> <eps> <mu> <thread_num> <num_pass> <num_warps> [log-file]
// num_warps sets the CTA size of the counting kernels (32 x num_warps threads);
// num_pass is accepted for compatibility: the whole graph stays resident in HBM,
// so the count needs no destination-range passes.
#include <stdio.h>
#include <stdlib.h>

#include <exception>

#include "scan_xp.h"

int main(int argc, char *argv[]) {
  if (argc < 5) {
    printf("Usage: [1]exe [2]graph-dir [3]similarity-threshold [4]density-threshold [5 thread_num] [6 num_pass] "
           "[7 num_warps] [8 optional]output\n");
    return 0;
  }
  double eps = strtod(argv[2], nullptr);
  int mu = atoi(argv[3]);
  int threads = atoi(argv[4]);
  int num_pass = argc > 5 ? atoi(argv[5]) : 1;
  int num_warps = argc > 6 ? atoi(argv[6]) : 0;
  if (argc > 7) accx_log_set_file(argv[7]);
  ScanXpOptions o = ScanXpOptions::from_env();
  if (num_warps > 0 && num_warps <= 32) o.block_warps = num_warps;
  (void)num_pass;
  try {
    SCAN_XP scanxp(threads, mu, eps, argv[1], o);
    scanxp.Execute();
  } catch (const std::exception &e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}

// CLI of the reference's scan-query-cuda/main_scanxp.cpp:14-40:
//   scan-xp-gb300 <graph-dir> <eps> <mu> <thread_num> [log-file]
#include <stdio.h>
#include <stdlib.h>

#include <exception>

#include "scan_xp.h"

int main(int argc, char *argv[]) {
  if (argc < 4) {
    printf("Usage: [1]exe [2]graph-dir [3]similarity-threshold [4]density-threshold [5 thread_num] [6 optional]output\n");
    return 0;
  }
  double eps = strtod(argv[2], nullptr);
  int mu = atoi(argv[3]);
  int threads = argc > 4 ? atoi(argv[4]) : 1;
  if (argc > 5) accx_log_set_file(argv[5]);
  try {
    SCAN_XP scanxp(threads, mu, eps, argv[1]);
    scanxp.Execute();
  } catch (const std::exception &e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}

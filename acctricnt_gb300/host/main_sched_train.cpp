// Trains the learned kernel scheduler on this GPU and writes its file:
//   accx-sched-train <out-file> [quick]
// SCAN_XP reads the file (ACCX_SCHED_MODEL, or accx-sched.model next to its
// executable) and counts with the scheduler's plan instead of the reference's
// ratio-50 rule.  "quick" trains on four small graphs (seconds; for tests).
#include <stdio.h>
#include <string.h>

#include "accx.h"

int main(int argc, char *argv[]) {
  if (argc < 2) {
    printf("Usage: %s <out-file> [quick]\n", argv[0]);
    return 0;
  }
  accx_sched_config c;
  memset(&c, 0, sizeof(c));
  c.quick = argc > 2 && strcmp(argv[2], "quick") == 0;
  accx_sched *s = nullptr;
  int rc = accx_sched_train(&c, &s);
  if (rc == ACCX_OK) rc = accx_sched_save(s, argv[1]);
  if (rc != ACCX_OK) {
    fprintf(stderr, "accx-sched-train: %s\n", accx_strerror(rc));
    if (s) accx_sched_free(s);
    return 1;
  }
  accx_sched_info in;
  accx_sched_get_info(s, &in);
  for (int o = 0; o < 2; o++)
    printf("%s model: %u rows, candidate %d of %d, loss %.3f -> %.3f, bitmap offset %.2f (collect %.1f s, train %.1f s, "
           "calibrate %.1f s)\n",
           o ? "oriented" : "direct", in.rows[o], in.chosen[o] + 1, in.candidates[o], in.loss_initial[o],
           in.loss_final[o], in.bitmap_offset[o], in.collect_s[o], in.train_s[o], in.calibrate_s[o]);
  printf("wrote %s\n", argv[1]);
  accx_sched_free(s);
  return 0;
}

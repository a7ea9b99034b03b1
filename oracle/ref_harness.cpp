// Dump harness for the reference's own CPU SCAN build (scan-query, BIT_VEC).
//
// TEST INFRASTRUCTURE ONLY: oracle/Makefile compiles this file together with the
// reference's scan-query sources, read in place from the reference tree, into
// oracle/_ref/ref_harness.  tests/golden/make_golden.py runs it to produce the
// fixtures that pin oracle/accx_oracle.c.  It replaces scan-query/main_scanxp.cpp
// (whose two globals it defines) and drives the same phases as
// SCAN_XP::Execute (scan-query/scan_xp.cpp:2076-2124), single-threaded because
// CheckCoreCompSimCore's core_count[u]++ is unsynchronised (scan_xp.cpp:124).
//
// usage: ref_harness <graph-dir> <eps> <mu> <dump-prefix>
// writes <prefix>.cnn (int32[m]), .sim (uint8[m]), .label (int32[n], final
// labels), .cluster (int32[n], min-id cluster of cores, -1 otherwise), and the
// reference's own <graph-dir>/scanxp-result-<eps>-<mu>.txt.
#include <cstdio>
#include <string>
#include <omp.h>
// Every standard header first, so the access override below reaches only the
// reference's SCAN_XP class declaration.
#include <bits/stdc++.h>
#if defined(__x86_64__)
#include <immintrin.h>
#endif
#define private public
#include "scan_xp.h"
#undef private

std::string reorder_method;
std::string dir;

static void dump(const std::string &path, const void *p, size_t bytes) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) { perror(path.c_str()); exit(2); }
  fwrite(p, 1, bytes, f);
  fclose(f);
}

int main(int argc, char *argv[]) {
  if (argc < 5) { fprintf(stderr, "usage: %s dir eps mu prefix\n", argv[0]); return 1; }
  omp_set_num_threads(1);
  double eps = strtod(argv[2], nullptr);
  int mu = atoi(argv[3]);
  std::string prefix = argv[4];
  dir = argv[1];
  reorder_method = "none";
  SCAN_XP s(1, mu, eps, argv[1]);
  s.CheckCore(&s.g);
  s.CheckCoreCompSimCore(&s.g);
  Graph &g = s.g;
  dump(prefix + ".cnn", g.common_node_num, sizeof(int) * (size_t)g.edgemax);
  std::vector<unsigned char> sim(g.edgemax);
  for (size_t e = 0; e < g.edgemax; e++) sim[e] = g.similarity[e] ? 1 : 0;
  dump(prefix + ".sim", sim.data(), sim.size());
  s.ClusterCore();
  s.LabelNonCore();
  s.PostProcess();
  s.PrepareResultOutput();
  dump(prefix + ".label", g.label, sizeof(int) * (size_t)g.nodemax);
  std::vector<int> cl(g.nodemax, -1);
  for (uint32_t i = 0; i < g.nodemax; i++)
    if (g.label[i] == CORE) cl[i] = g.cluster_dict[s.uf_ptr->FindRoot(i)];
  dump(prefix + ".cluster", cl.data(), sizeof(int) * cl.size());
  return 0;
}

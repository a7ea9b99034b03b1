// Harness for the reference's multi-GPU vertex partitioner.
//
// TEST INFRASTRUCTURE ONLY: oracle/Makefile compiles this file with nvcc, which
// includes scan-query-cuda/scan_xp_multi_gpu_multi_pass_common.cu in place from
// the reference tree (nothing is copied), into oracle/_ref/ref_ranges.
// tests/golden/make_golden.py runs it to record the reference's own
// ComputeVertexRangeAccumulatedFilteredDegree
// (scan-query-cuda/scan_xp_multi_gpu_multi_pass_common.cu:516-554) ranges, which
// pin the oracle's and the library's partitioner.  Only that host function is
// called: the harness defines the Graph constructor (its own reader of
// b_degree.bin / b_adj.bin) and empty bodies for the two members the included
// file refers to but this program never calls.
//
// usage: ref_ranges <graph-dir> <parts>...   prints one line of parts+1 ids per count
#include "scan_xp_multi_gpu_multi_pass_common.cu"

#include <cstdio>
#include <cstdlib>

Graph::Graph(char *dir_cstr) {
  dir = dir_cstr;
  nodemax = edgemax = 0;
  node_off = nullptr;
  edge_dst = nullptr;
  FILE *f = fopen((dir + "/b_degree.bin").c_str(), "rb");
  int int_size = 0;
  if (!f || fread(&int_size, 4, 1, f) != 1 || fread(&nodemax, 4, 1, f) != 1 || fread(&edgemax, 4, 1, f) != 1) {
    fprintf(stderr, "cannot read %s/b_degree.bin\n", dir_cstr);
    exit(2);
  }
  std::vector<int> deg(nodemax);
  if (nodemax && fread(deg.data(), 4, nodemax, f) != nodemax) exit(2);
  fclose(f);
  node_off = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)nodemax + 1));
  edge_dst = (int *)malloc(sizeof(int) * ((size_t)edgemax + 1));
  node_off[0] = 0;
  for (uint32_t i = 0; i < nodemax; i++) node_off[i + 1] = node_off[i] + (uint32_t)deg[i];
  f = fopen((dir + "/b_adj.bin").c_str(), "rb");
  if (!f || (edgemax && fread(edge_dst, 4, edgemax, f) != edgemax)) {
    fprintf(stderr, "cannot read %s/b_adj.bin\n", dir_cstr);
    exit(2);
  }
  fclose(f);
}

void Graph::Output(const char *, const char *, UnionFind *) {}
void SCAN_XP::CheckCore(Graph *) {}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s <graph-dir> <parts>...\n", argv[0]);
    return 1;
  }
  Graph g(argv[1]);
  for (int a = 2; a < argc; a++) {
    std::vector<int32_t> r = ComputeVertexRangeAccumulatedFilteredDegree(&g, atoi(argv[a]));
    for (size_t i = 0; i < r.size(); i++) printf("%s%d", i ? " " : "", r[i]);
    printf("\n");
  }
  return 0;
}

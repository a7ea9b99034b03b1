// CLI of the reference's edge-list converter (scan-query/converter/EdgeListToBinsConverter.cpp:24-160):
//   edge-list-to-bins-gb300 <edge-list.txt> <b_degree.bin> <b_adj.bin>
//
// Reads a text edge list the way the reference does -- lines starting with '#'
// are comments, each other line holds two vertex ids, and only lines with
// first < second are kept (a self loop or a reversed copy of an edge is dropped)
// -- sets n to the largest kept id + 1, and builds the symmetric CSR on the GPU
// (accx_graph_from_edges: both directions, repeated edges once, rows sorted).
// The two files are the reference's format: b_degree.bin = int32 4, uint32 n,
// uint32 entry count, int32 degree[n]; b_adj.bin = int32 neighbour ids row by row.
//
// Differences, all on malformed input only: a repeated edge is counted once in
// the degree file as in the adjacency file (the reference counts every copy in
// the degrees but writes one adjacency entry); a line without two numbers (a
// blank line) is skipped (the reference reads uninitialised ids for it); a last
// line without a trailing newline is read (the reference's read loop stops
// before it).
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "accx.h"

using clk = std::chrono::steady_clock;

static double ms_since(clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); }

// Parses `buf` (len bytes) into kept edges; returns false on an id out of range.
static bool parse_edges(const char *buf, size_t len, std::vector<uint32_t> &src, std::vector<uint32_t> &dst,
                        int64_t &max_id) {
  size_t i = 0;
  while (i < len) {
    size_t e = i;
    while (e < len && buf[e] != '\n') e++;
    if (buf[i] != '#') {
      int64_t v[2];
      int got = 0;
      size_t p = i;
      while (got < 2 && p < e) {
        while (p < e && (buf[p] == ' ' || buf[p] == '\t' || buf[p] == '\r')) p++;
        if (p >= e) break;
        bool neg = false;
        if (buf[p] == '-' || buf[p] == '+') neg = buf[p++] == '-';
        if (p >= e || buf[p] < '0' || buf[p] > '9') break;
        int64_t x = 0;
        while (p < e && buf[p] >= '0' && buf[p] <= '9') {
          x = x * 10 + (buf[p++] - '0');
          if (x > INT32_MAX) return false;
        }
        v[got++] = neg ? -x : x;
      }
      if (got == 2 && v[0] < v[1]) {
        if (v[0] < 0) return false;
        src.push_back((uint32_t)v[0]);
        dst.push_back((uint32_t)v[1]);
        if (v[1] > max_id) max_id = v[1];
      }
    }
    i = e + 1;
  }
  return true;
}

static bool write_file(const char *path, const void *a, size_t na, const void *b, size_t nb) {
  FILE *f = fopen(path, "wb");
  if (!f) return false;
  bool ok = (na == 0 || fwrite(a, 1, na, f) == na) && (nb == 0 || fwrite(b, 1, nb, f) == nb);
  return fclose(f) == 0 && ok;
}

int main(int argc, char *argv[]) {
  if (argc < 4) {
    printf("Usage: [1]exe [2]edge-list-file [3]degree-output-file [4]adjacency-output-file\n");
    return 1;
  }
  auto t0 = clk::now();
  FILE *f = fopen(argv[1], "rb");
  if (!f) {
    fprintf(stderr, "cannot read %s\n", argv[1]);
    return 1;
  }
  std::vector<char> buf;
  char chunk[1 << 16];
  size_t got;
  while ((got = fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  fclose(f);
  std::vector<uint32_t> src, dst;
  int64_t max_id = -1;
  if (!parse_edges(buf.data(), buf.size(), src, dst, max_id)) {
    fprintf(stderr, "vertex id out of range (0 .. 2^31-1)\n");
    return 1;
  }
  printf("1st, read file and parse string cost:%.0f ms\n", ms_since(t0));
  printf("max vertex id:%lld\n", (long long)max_id);
  printf("number of edges:%zu\n", src.size());
  const uint32_t n = (uint32_t)(max_id + 1);
  std::vector<uint32_t> off(n + 1, 0);
  std::vector<int32_t> adj;
  auto t1 = clk::now();
  if (n > 0) {
    accx_graph *g = nullptr;
    int rc = accx_graph_from_edges(src.data(), dst.data(), src.size(), n, nullptr, &g);
    if (rc) {
      fprintf(stderr, "accx_graph_from_edges: %s\n", accx_strerror(rc));
      return 1;
    }
    uint32_t gn = 0;
    uint64_t m = 0;
    accx_graph_size(g, &gn, &m);
    adj.resize(m);
    rc = accx_graph_download(g, off.data(), adj.data(), nullptr);
    accx_graph_free(g);
    if (rc) {
      fprintf(stderr, "accx_graph_download: %s\n", accx_strerror(rc));
      return 1;
    }
  }
  const uint64_t m = adj.size();
  if (m >= (1ull << 32)) {
    fprintf(stderr, "%llu entries exceed the format's 32-bit count\n", (unsigned long long)m);
    return 1;
  }
  std::vector<int32_t> head(3 + (size_t)n);
  head[0] = (int32_t)sizeof(int32_t);
  uint32_t n32 = n, m32 = (uint32_t)m;
  memcpy(&head[1], &n32, 4);
  memcpy(&head[2], &m32, 4);
  for (uint32_t u = 0; u < n; u++) head[3 + u] = (int32_t)(off[u + 1] - off[u]);
  if (!write_file(argv[2], head.data(), head.size() * 4, nullptr, 0) ||
      !write_file(argv[3], adj.data(), adj.size() * 4, nullptr, 0)) {
    fprintf(stderr, "cannot write the output files\n");
    return 1;
  }
  printf("3rd, construct csr (GPU) and write file cost:%.0f ms\n", ms_since(t1));
  return 0;
}

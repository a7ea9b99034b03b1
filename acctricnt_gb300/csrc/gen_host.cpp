// Host generator: the same counter-based edge streams as the device generator
// (gen.cu), symmetrised, with self loops and duplicates removed, sorted into a
// CSR.  Used by tests and to write graph files in the reference format.
#include "gen_host.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

int accx_gen_shape(const accx_gen_params *p, uint32_t *n, uint64_t *draws) {
  if (!p) return ACCX_ERR_INVALID_ARG;
  switch (p->kind) {
    case ACCX_GEN_RMAT:
      if (p->p0 < 1 || p->p0 > 31 || p->p1 < 1) return ACCX_ERR_INVALID_ARG;
      if (!(p->q0 >= 0 && p->q1 >= 0 && p->q2 >= 0 && p->q0 + p->q1 + p->q2 <= 1.0)) return ACCX_ERR_INVALID_ARG;
      *n = (uint32_t)(1ull << p->p0);
      *draws = p->p1 << p->p0;
      break;
    case ACCX_GEN_ER:
    case ACCX_GEN_CHUNG_LU:
      if (p->p0 < 1 || p->p0 > 0x7fffffffull || p->p1 < 1) return ACCX_ERR_INVALID_ARG;
      if (p->kind == ACCX_GEN_CHUNG_LU && !(p->q0 > 1.0 && p->q1 >= 1.0)) return ACCX_ERR_INVALID_ARG;
      *n = (uint32_t)p->p0;
      *draws = p->p1;
      break;
    default:
      return ACCX_ERR_INVALID_ARG;
  }
  // Two directed entries per draw must stay below the 32-bit entry count of the format.
  if (*draws >= (1ull << 31)) return ACCX_ERR_TOO_LARGE;
  return ACCX_OK;
}

accx_rmat_thresholds accx_rmat_make(double a, double b, double c) {
  const double s = 9007199254740992.0;  // 2^53
  accx_rmat_thresholds t;
  t.ta = (uint64_t)floor(a * s);
  t.tab = (uint64_t)floor((a + b) * s);
  t.tabc = (uint64_t)floor((a + b + c) * s);
  return t;
}

// Sum_{i=0}^{n-1} (i + i0)^(-alpha): exact over the first terms, midpoint
// integral for the tail (only used to pick i0).
static double cl_weight_sum(uint32_t n, double i0, double alpha) {
  const uint32_t K = n < 4096 ? n : 4096;
  double s = 0;
  for (uint32_t i = 0; i < K; i++) s += pow(i + i0, -alpha);
  if (K < n) {
    double a = K - 0.5 + i0, b = n - 0.5 + i0;
    s += (pow(b, 1 - alpha) - pow(a, 1 - alpha)) / (1 - alpha);
  }
  return s;
}

void accx_chung_lu_cdf(uint32_t n, uint64_t draws, double gamma, double max_deg, std::vector<uint64_t> &cdf) {
  double alpha = 1.0 / (gamma - 1.0);
  // expected degree of vertex 0 = 2 * draws * i0^-alpha / W(i0); decreasing in i0.
  double lo = 1e-6, hi = (double)n + 1.0;
  for (int it = 0; it < 200; it++) {
    double mid = sqrt(lo * hi);
    double d0 = 2.0 * (double)draws * pow(mid, -alpha) / cl_weight_sum(n, mid, alpha);
    if (d0 > max_deg) lo = mid; else hi = mid;
  }
  double i0 = sqrt(lo * hi);
  std::vector<double> w(n);
  double total = 0;
  for (uint32_t i = 0; i < n; i++) {
    w[i] = pow(i + i0, -alpha);
    total += w[i];
  }
  cdf.assign((size_t)n + 1, 0);
  const double scale = 4611686018427387904.0;  // 2^62
  double acc = 0;
  for (uint32_t i = 0; i < n; i++) {
    acc += w[i];
    double c = acc / total * scale;
    uint64_t ci = c >= scale ? (1ull << 62) : (uint64_t)c;
    cdf[i + 1] = ci < cdf[i] ? cdf[i] : ci;
  }
  cdf[n] = 1ull << 62;
}

static void gen_keys(const accx_gen_params *p, uint32_t n, uint64_t draws, std::vector<uint64_t> &keys) {
  uint64_t seed_mix = accx_mix64(p->seed);
  keys.clear();
  keys.reserve(draws * 2);
  std::vector<uint64_t> cdf;
  accx_rmat_thresholds t{};
  if (p->kind == ACCX_GEN_RMAT) t = accx_rmat_make(p->q0, p->q1, p->q2);
  if (p->kind == ACCX_GEN_CHUNG_LU) accx_chung_lu_cdf(n, draws, p->q0, p->q1, cdf);
  for (uint64_t k = 0; k < draws; k++) {
    uint32_t u, v;
    if (p->kind == ACCX_GEN_RMAT) accx_rmat_edge(seed_mix, k, (int)p->p0, t, &u, &v);
    else if (p->kind == ACCX_GEN_ER) accx_er_edge(seed_mix, k, n, &u, &v);
    else accx_cl_edge(seed_mix, k, cdf.data(), n, &u, &v);
    if (u == v) continue;
    keys.push_back(((uint64_t)u << 32) | v);
    keys.push_back(((uint64_t)v << 32) | u);
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
}

extern "C" int accx_generate_host(const accx_gen_params *p, uint32_t *n_out, uint64_t *m_out, uint32_t *off,
                                  int32_t *dst) {
  if (!p || !n_out || !m_out) return ACCX_ERR_INVALID_ARG;
  uint32_t n;
  uint64_t draws;
  int rc = accx_gen_shape(p, &n, &draws);
  if (rc) return rc;
  std::vector<uint64_t> keys;
  gen_keys(p, n, draws, keys);
  *n_out = n;
  *m_out = keys.size();
  if (!off || !dst) return ACCX_OK;
  std::fill(off, off + (size_t)n + 1, 0u);
  for (uint64_t i = 0; i < keys.size(); i++) {
    off[(keys[i] >> 32) + 1]++;
    dst[i] = (int32_t)(keys[i] & 0xffffffffu);
  }
  for (uint32_t i = 0; i < n; i++) off[i + 1] += off[i];
  return ACCX_OK;
}

// Host-side parts of the synthetic generators (shared by the host generator and
// the device generator, which uploads the Chung-Lu table built here).
#pragma once
#include <stdint.h>

#include <vector>

#include "../../include/accx.h"
#include "gen_rng.h"

// Number of vertices and of edge draws for a parameter set; ACCX_ERR_* on bad input.
int accx_gen_shape(const accx_gen_params *p, uint32_t *n, uint64_t *draws);

// R-MAT thresholds from (a, b, c).
accx_rmat_thresholds accx_rmat_make(double a, double b, double c);

// Chung-Lu cumulative weight table cdf[0..n], cdf[n] = 2^62, with expected
// degree w_i proportional to (i + i0)^(-1/(gamma-1)) and i0 chosen so that the
// expected degree of vertex 0 is max_deg.
void accx_chung_lu_cdf(uint32_t n, uint64_t draws, double gamma, double max_deg, std::vector<uint64_t> &cdf);

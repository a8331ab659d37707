/*
 * sgs_oracle.h — FP64 CPU oracle for sequential Gaussian simulation.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA library is compared
 * against (tests/, __graft_entry__.smoke(), bench.py's CPU baseline leg); the
 * product path never links, loads or calls it.
 *
 * It restates GeoStatsProcesses.jl v0.13.0's SEQSIM for a GaussianProcess
 * (src/simulation/field/seqsim.jl:50-156) with one simulation path shared by
 * all realizations, so the realization-independent search and kriging solve
 * are computed once and the draw loop runs per realization.  The upstream
 * steps the reference delegates to packages that are not vendored
 * (Meshes.KBallSearch/KNearestSearch, GeoStatsFunctions variograms,
 * GeoStatsModels simple kriging, LAPACK Cholesky) are restated from their
 * published definitions; the canonical neighbour order (FP64 distance, then
 * augmented point index) and the singular-pivot rule are this project's
 * definitions, documented in oracle/sgs_oracle.cpp.
 *
 * Parity status: partially pinned.  The reference's own known-answer tests
 * for this path (test/field.jl:86 data reproduction, test/initialization.jl
 * :31-59 ExplicitInit placement) are reproduced in tests/; neighbour order,
 * weights and values are pinned against closed-form kriging systems and an
 * independent numpy restatement (tests/golden/make_golden.py), not against
 * reference outputs (Julia is not available to run the reference).
 */
#ifndef SGS_ORACLE_H
#define SGS_ORACLE_H

#include <stdint.h>
#include "../include/geosgs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_plan oracle_plan;

#define ORACLE_SEARCH_BRUTE    0  /* scan every cell of the neighbourhood's bounding box, sort */
#define ORACLE_SEARCH_TEMPLATE 1  /* scan the offset template in canonical order */

int  oracle_create(const sgs_problem* problem, oracle_plan** plan);
void oracle_destroy(oracle_plan* plan);
const char* oracle_last_error(void);

/* Neighbour search for path ranks t in [t_begin, t_end) with step `stride`. */
int oracle_search(oracle_plan* plan, int method, int64_t t_begin, int64_t t_end,
                  int64_t stride, int nthreads);
/* Kriging build + Cholesky + weights for the same rank selection. */
int oracle_solve(oracle_plan* plan, int64_t t_begin, int64_t t_end, int64_t stride,
                 int nthreads);
/* Draw loop over path ranks [0, t_end) for nreals realizations (OpenMP over
 * realizations).  z: nreals x N realization-major or NULL (seeded Philox
 * draws, oracle_normals).  out: nreals x N realization-major. */
int oracle_simulate(oracle_plan* plan, int32_t nreals, const double* z, uint64_t seed,
                    double* out, int64_t t_end, int nthreads);

/* Sequential indicator simulation on the prepared plan: ncat categories,
 * prior probabilities prob, data categories data_cat (D); u: nreals x N
 * uniforms or NULL (oracle_uniforms of seed); out: nreals x N categories. */
int oracle_simulate_indicator(oracle_plan* plan, int32_t ncat, const double* prob, const int32_t* data_cat,
                              int32_t nreals, const double* u, uint64_t seed, int32_t* out, int nthreads);
/* Sequential indicator simulation with full simple cokriging for an
 * indicator covariance that is a linear model of coregionalization:
 * C_ab(h) = sum_s coef[s][a][b] C_s(h) over the structures of the plan's
 * (nested) variogram; coef: S x ncat x ncat row-major, S = 1 + nstructures.
 * Requires maxneighbors x ncat <= 64.  Node status is left in the plan. */
int oracle_simulate_cokriging(oracle_plan* plan, int32_t ncat, const double* prob, const int32_t* data_cat,
                              const double* coef, int32_t nreals, const double* u, uint64_t seed, int32_t* out,
                              int nthreads);
/* Uniforms of the seeded indicator draws: u[r*nnodes + g]. */
void oracle_uniforms(uint64_t seed, int64_t nnodes, int32_t nreals, double* u);

/* Posterior mean and variance by simple kriging from the data alone, every
 * grid node (NaN where the reference's prediction is missing). */
int oracle_krige(oracle_plan* plan, double* mean, double* var, int nthreads);

int oracle_neighbors(const oracle_plan* plan, int32_t* idx, int32_t* count);
int oracle_weights(const oracle_plan* plan, double* weights, double* sigma, int32_t* status);
int oracle_levels(const oracle_plan* plan, int32_t* level, int32_t* nlevels);
int oracle_template_size(const oracle_plan* plan);

/* Standard normals of the seeded mode: z[r*nnodes + g] for r < nreals. */
void oracle_normals(uint64_t seed, int64_t nnodes, int32_t nreals, double* z);

/* Covariance C(lag) = sill - gamma(lag) of a variogram (test helper). */
double oracle_covariance(const sgs_variogram* v, int32_t dim, const double* lag);

#ifdef __cplusplus
}
#endif

#endif

/*
 * Oracle: CPU restatement of Abeille's multigroup transport loop.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load this library, and only as the
 * checker or the CPU baseline; the product path never calls it.
 *
 * It restates, function by function, the reference's algorithm on the same
 * flattened problem the product takes (include/abeille_gb300.h), and is
 * compiled with -ffp-contract=off so that no FMA contraction changes the
 * reference's rounding.  The reference cannot be built here (it needs yaml-cpp,
 * PapillonNDL, HighFive, NDArray, docopt and Boost.unordered, none of which are
 * present); its third-party arithmetic (pcg-cpp's pcg32 and libstdc++'s
 * <random> distributions) is pinned by golden vectors generated from the real
 * libraries (tests/golden/make_rng_golden.py).
 */
#ifndef ABX_ORACLE_H
#define ABX_ORACLE_H

#include "../include/abeille_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

const char* oracle_last_error(void);

int oracle_create(const abx_problem* problem, oracle_ctx** out);
void oracle_destroy(oracle_ctx* ctx);

int oracle_sample_sources(oracle_ctx* ctx, uint64_t first_history_id, size_t n,
                          abx_particle* out);
int oracle_transport(oracle_ctx* ctx, const abx_particle* bank, size_t n,
                     double kcol, int converged, abx_site* sites,
                     size_t site_capacity, size_t* n_sites, abx_scores* scores,
                     int nthreads);
int oracle_tally_record_generation(oracle_ctx* ctx, double multiplier);
int oracle_tally_clear_generation(oracle_ctx* ctx);
int oracle_tally_size(oracle_ctx* ctx, int id, size_t* n_bins);
int oracle_tally_read(oracle_ctx* ctx, int id, double* gen, double* avg,
                      double* var, int* generations);
int oracle_entropy(oracle_ctx* ctx, const abx_site* sites, size_t n,
                   double* entropy);
int oracle_run_power_iteration(oracle_ctx* ctx, int ngenerations, int nignored,
                               int nthreads, abx_run_stats* stats,
                               double* kcol_per_gen, double* entropy_per_gen);
int oracle_set_source_bank(oracle_ctx* ctx, const double* source, size_t n);
void oracle_shuffle(void* data, size_t n, size_t elem_size, uint64_t* state);
int oracle_run_fixed_source(oracle_ctx* ctx, int nbatches, uint64_t nparticles,
                            int nthreads, abx_run_stats* stats);
int oracle_set_trace(oracle_ctx* ctx, uint32_t n_hist, size_t capacity);
int oracle_get_trace(oracle_ctx* ctx, abx_trace_rec* out, size_t capacity,
                     size_t* n_out);

/* Derived tables, exported so tests can compare them with the product's. */
int oracle_majorant(oracle_ctx* ctx, double* out /* [ngroups] */);
int oracle_scatter_cdf(oracle_ctx* ctx, int mat, int g, double* out /* [G] */);

/* RNG primitives (golden-vector tests). */
void oracle_pcg32_seed(uint64_t seed, uint64_t* state);
uint32_t oracle_pcg32_next(uint64_t* state);
void oracle_pcg32_advance(uint64_t* state, uint64_t delta);
double oracle_canonical(uint64_t* state);
double oracle_exponential(uint64_t* state, double lambda);
int oracle_discrete(uint64_t* state, const double* weights, int n);

#ifdef __cplusplus
}
#endif

#endif

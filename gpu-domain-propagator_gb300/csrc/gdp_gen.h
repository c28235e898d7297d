/*
 * gdp_gen.h -- seeded synthetic MIP generators (host C++, libgdpgen.so).
 *
 * The reference benchmarks on MIPLIB 2017 instances; seeded synthetic MIPs
 * with the row-length skew, coefficient ranges, integrality mix and infinite
 * bounds of those instances stand in for them. The same generated instance is
 * fed to the GPU library and to the CPU oracle/baseline. Random numbers come
 * from this file's own xoshiro256** streams (one per block of rows), so an
 * instance depends only on (parameters, seed), not on the thread count.
 */
#ifndef GDP_GEN_H
#define GDP_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int m, n, nnz;
    int *row_ptr;     /* m+1 */
    int *col;         /* nnz, ascending within each row */
    double *val;      /* nnz */
    double *lhs;      /* m (-1e20 = -inf) */
    double *rhs;      /* m (+1e20 = +inf) */
    double *lb;       /* n */
    double *ub;       /* n */
    int *vartype;     /* n: 0 binary, 1 integer, 3 continuous */
    double *x0;       /* n: the hidden feasible point */
} gdp_instance;

/* Random MIP with a hidden feasible point x0. */
typedef struct {
    int m, n;
    int len_dist;        /* 0: uniform {len_min..len_max}; 1: Zipf(zipf_s) clipped to [len_min, len_max] */
    int len_min, len_max;
    double zipf_s;
    int n_dense_rows, dense_len;   /* extra long rows (placed at random row positions) */
    int coef_dist;       /* 0: +-U[coef_min, coef_max]; 1: +-LogUniform[coef_min, coef_max] */
    double coef_min, coef_max;
    double frac_int_coef;          /* fraction of coefficients rounded to a non-zero integer */
    double frac_int_vars;          /* integer vars with bounds [0, U{1..int_ub_max}] */
    int int_ub_max;
    double frac_inf_vars;          /* continuous vars with one infinite bound */
    double cont_bound_max;         /* continuous bounds [-U[1,B], U[1,B]] */
    double slack_max;              /* lhs = A x0 - U[0,slack_max]*len, rhs = A x0 + U[0,slack_max]*len */
    double frac_one_sided;         /* rows with lhs = -inf (of the non-equality rows) */
    double frac_equality;          /* rows with lhs = rhs = A x0 */
    uint64_t seed;
} gdp_gen_params;

/* Fills *p with the parameters of the named workload:
 *   0: small random MIP (m=2,000, n=1,500, row length U{2..16})
 *   1: large power-law MIP (m=2,000,000, n=1,500,000, Zipf(1.8) rows in
 *      [2, 20,000] plus 32 rows of 100,000 non-zeros, 30% equality rows)
 * m/n may be rescaled afterwards by the caller. Returns 0 or -1. */
int gdp_gen_default_params(int workload, gdp_gen_params *p);

/* Generates an instance; arrays are malloc'ed and released by gdp_gen_free.
 * Returns 0 on success, <0 on bad parameters or allocation failure. */
int gdp_gen_random_mip(const gdp_gen_params *p, gdp_instance *out);

/* Set-covering rows (0/1 coefficients, length U{cover_min..cover_max},
 * lhs = 1) over n_bin binary vars, plus knapsack rows (integer coefficients
 * U{1..1000}, capacity 0.3 * row sum) over binary and n_cont continuous vars
 * in [0, U[1,10]]. Feasible by construction (x0 covers every row). */
int gdp_gen_cover_knapsack(int n_cover_rows, int n_knap_rows, int n_bin, int n_cont,
                           int cover_min, int cover_max, int knap_min, int knap_max,
                           uint64_t seed, gdp_instance *out);

/* Chains x_{i+1} - x_i <= c_i (c_i ~ U[0,3], chains up to chain_max long)
 * mixed 50/50 by rows with power-law rows of the large random MIP (over
 * other variables; frac_equality of them equality rows, 0.3 in the large
 * MIP); when make_infeasible != 0 one chain's end gets a lower bound above
 * what the chain allows, by at least 1. */
int gdp_gen_chains(int m, int n, int chain_max, double frac_int_vars, double frac_inf_vars,
                   double frac_equality, int make_infeasible, uint64_t seed, gdp_instance *out);

void gdp_gen_free(gdp_instance *inst);

#ifdef __cplusplus
}
#endif

#endif

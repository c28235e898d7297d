/*
 * gdp_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference propagation math, used as the checker for
 * the GPU path: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it. The product library never links or calls it.
 *
 * Parity is pinned: tests check this restatement against the reference's own
 * analytical fixtures (test/test_setups.cuh) and, in the build container,
 * bit-for-bit against the reference's cpu_seq / cpu_omp round functions
 * compiled from the reference sources (oracle/ref_harness.cpp, oracle/_ref/).
 */
#ifndef GDP_ORACLE_H
#define GDP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Schedules. JACOBI reads the round-start snapshot of the bounds and applies,
 * per variable, the max (lb) / min (ub) of every candidate that is EPS-better
 * than the snapshot: the reference's OMPPropagationRound
 * (src/propagators/OMP_propagator.h:10-137) with its "apply if better"
 * lock section made order-independent. SEQUENTIAL is Gauss-Seidel in row
 * order with in-place updates: the reference's sequentialPropagationRound
 * (src/propagators/sequential_propagator.h:13-123). */
enum { GDPO_SCHED_JACOBI = 0, GDPO_SCHED_SEQUENTIAL = 1 };

typedef struct {
    double minact, maxact, maxactdelta;
    int minact_inf, maxact_inf;
} gdpo_acts;

typedef struct {
    int rounds;          /* rounds executed (the reference's prop_round - 1) */
    int converged;       /* 1 if the last executed round found no change */
    int infeasible;      /* 1 if the infeasibility rule fired */
    int infeasible_var;  /* first variable index violating it, or -1 */
    long long candidates;  /* bound tightenings found (summed over rounds) */
    long long rows_processed; /* marked rows processed (summed over rounds) */
    long long nnz_processed;  /* their non-zeros */
    long long rows_go;        /* GPU mode: processed rows of at most split_tile non-zeros that passed
                                 their row test (summed over rounds) */
    int infeasible_row;       /* smallest row found infeasible by the row rule in the last round, or -1 */
} gdpo_result;

/* --- reference math, one function each (known-answer tests call these) --- */
double gdpo_adjust_upper(int is_cont, double ub);
double gdpo_adjust_lower(int is_cont, double lb);
int gdpo_is_lb_better(double lb, double ub, double newlb);
int gdpo_is_ub_better(double lb, double ub, double newub);
int gdpo_can_cons_be_tightened(double minact, double maxact, int minact_inf, int maxact_inf,
                               double lhs, double rhs, double maxactdelta);
int gdpo_is_cons_infeasible(double minact, double maxact, double rhs, double lhs);
/* returns is_tightened; *newb receives the bound (old one if not tightened) */
int gdpo_tighten_var_upper(double coeff, double slack, double surplus, int num_inf,
                           double lb, double ub, int is_cont, double *newb);
int gdpo_tighten_var_lower(double coeff, double slack, double surplus, int num_inf,
                           double lb, double ub, int is_cont, double *newb);
void gdpo_tighten_variable(double coeff, double lhs, double rhs, double minact, double maxact,
                           int minact_inf, int maxact_inf, int is_cont, double lb, double ub,
                           int *lb_tightened, double *newlb, int *ub_tightened, double *newub);
gdpo_acts gdpo_activities(int row, const int *col, const int *row_ptr, const double *val,
                          const double *lb, const double *ub);
/* infeasibility rules applied in every round: variable crossing (after the
 * round) and the row rule (every processed row, on the activities it computed) */
int gdpo_var_infeasible(double lb, double ub);
int gdpo_row_infeasible(double minact, double maxact, int minf, int maxf, double lhs, double rhs);

/* --- full propagation to a fixpoint ---
 * lb/ub in/out. max_rounds <= 0 means the reference cap (100). nthreads > 1
 * runs the JACOBI schedule with OpenMP threads (result independent of the
 * thread count). row_round_tightened (optional, length m) receives for each
 * row the last round in which it produced a tightening (0 if never): used by
 * the trace tests of learned marking. Returns 0 on success, <0 on bad input. */
int gdpo_propagate(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                   const double *lhs, const double *rhs, double *lb, double *ub,
                   const int *vartype, int schedule, int max_rounds, int nthreads,
                   gdpo_result *res);

/* gdpo_propagate in GPU mode when split_tile > 0 (JACOBI schedule): rows
 * longer than split_len (the kernels' thread_row_max) are summed in the GB300
 * kernels' lane-group / warp-tile order with split_tile non-zeros per tile
 * (see gdp_oracle.c); the row test and candidates stay the reference's.
 * split_tile = 0 is the reference mode (identical to gdpo_propagate). */
int gdpo_propagate_ex(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                      const double *lhs, const double *rhs, double *lb, double *ub,
                      const int *vartype, int schedule, int max_rounds, int nthreads,
                      int split_len, int split_tile, gdpo_result *res);
/* lanes per row the GPU mode uses for a row of len non-zeros */
int gdpo_lanes_per_row(int len, int thread_row_max, int tile);

/* One JACOBI round on a snapshot, restricted to rows with mark[row] != 0
 * (mark == NULL: every row). Writes candidates into lb_out/ub_out (which must
 * hold a copy of lb/ub on entry) and sets tight_row[row] = 1 for every row
 * that produced a tightening (optional). Returns 1 if any tightening. */
int gdpo_jacobi_round(int m, int n, const int *col, const int *row_ptr, const double *val,
                      const double *lhs, const double *rhs, const double *lb, const double *ub,
                      const int *vartype, const unsigned char *mark, double *lb_out,
                      double *ub_out, unsigned char *tight_row, int nthreads);

#ifdef __cplusplus
}
#endif

#endif

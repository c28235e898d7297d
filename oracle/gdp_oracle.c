/*
 * gdp_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * Plain-C restatement of the reference's CPU propagation, used as the checker
 * of the GPU path by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg. Nothing in the product library links, loads or calls it.
 *
 * Each function names the reference file:line it restates. Compile with
 * -ffp-contract=off: the reference's x86 build never fuses a*b+c, and every
 * expression here must round exactly like the reference's.
 */
#include "gdp_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_INF 1e20
#define O_EPS 1e-9
#define O_FEASTOL 1e-6
#define O_MAX_ROUNDS 100

/* EPS comparisons: reference src/def.h:68-79 */
static inline int eps_le(double x, double y) { return (x - y) <= O_EPS; }
static inline int eps_lt(double x, double y) { return (x - y) < -O_EPS; }
static inline int eps_ge(double x, double y) { return (x - y) >= -O_EPS; }
static inline int eps_gt(double x, double y) { return (x - y) > O_EPS; }
static inline double eps_floor(double x) { return floor(x + O_EPS); }
static inline double eps_ceil(double x) { return ceil(x - O_EPS); }
static inline int is_posinf(double x) { return eps_ge(x, O_INF); }
static inline int is_neginf(double x) { return eps_le(x, -O_INF); }
/* std::min(a, b) as the reference's canConsBeTightened uses it */
static inline double std_min(double a, double b) { return (b < a) ? b : a; }

/* reference src/propagation_methods.cuh:40-47 */
double gdpo_adjust_upper(int is_cont, double ub) { return is_cont ? ub : eps_floor(ub); }
/* reference src/propagation_methods.cuh:49-52 */
double gdpo_adjust_lower(int is_cont, double lb) { return is_cont ? lb : eps_ceil(lb); }
/* reference src/propagation_methods.cuh:54-58 (the assert is a debug check only) */
int gdpo_is_lb_better(double lb, double ub, double newlb) { (void)ub; return eps_gt(newlb, lb); }
/* reference src/propagation_methods.cuh:60-64 */
int gdpo_is_ub_better(double lb, double ub, double newub) { (void)lb; return eps_lt(newub, ub); }

/* reference src/propagation_methods.cuh:136-154 */
int gdpo_can_cons_be_tightened(double minact, double maxact, int minact_inf, int maxact_inf,
                               double lhs, double rhs, double maxactdelta) {
    if (minact_inf > 1 && maxact_inf > 1) return 0;
    if (eps_lt(maxactdelta, O_INF)) return !eps_le(maxactdelta, std_min(rhs - minact, maxact - lhs));
    return 1;
}

/* reference src/propagation_methods.cuh:156-159 */
int gdpo_is_cons_infeasible(double minact, double maxact, double rhs, double lhs) {
    return (minact > rhs || maxact < lhs);
}

/* Row-side infeasibility rule of this project (the reference never calls
 * isConsInfeasible on a propagation path): the reference's isConsInfeasible
 * (src/propagation_methods.cuh:156-159), taken only on a side with a finite
 * constraint side and no infinite contribution, with the relative tolerance
 * of gdpo_var_infeasible. */
int gdpo_row_infeasible(double minact, double maxact, int minf, int maxf, double lhs, double rhs) {
    if (minf == 0 && !is_posinf(rhs)) {
        double s = fabs(minact) > fabs(rhs) ? fabs(minact) : fabs(rhs);
        if (s < 1.0) s = 1.0;
        if (minact - rhs > O_FEASTOL * s) return 1;
    }
    if (maxf == 0 && !is_neginf(lhs)) {
        double s = fabs(maxact) > fabs(lhs) ? fabs(maxact) : fabs(lhs);
        if (s < 1.0) s = 1.0;
        if (lhs - maxact > O_FEASTOL * s) return 1;
    }
    return 0;
}

/* reference src/propagation_methods.cuh:78-106 */
int gdpo_tighten_var_upper(double coeff, double slack, double surplus, int num_inf,
                           double lb, double ub, int is_cont, double *newb_out) {
    double newb;
    *newb_out = ub;
    if (num_inf == 0) {
        newb = coeff > 0 ? slack / coeff : surplus / coeff;
        newb += lb;
    } else if (num_inf == 1 && is_neginf(lb)) {
        newb = coeff > 0 ? slack / coeff : surplus / coeff;
    } else {
        return 0;
    }
    newb = gdpo_adjust_upper(is_cont, newb);
    if (gdpo_is_ub_better(lb, ub, newb)) {
        *newb_out = newb;
        return 1;
    }
    return 0;
}

/* reference src/propagation_methods.cuh:108-134 */
int gdpo_tighten_var_lower(double coeff, double slack, double surplus, int num_inf,
                           double lb, double ub, int is_cont, double *newb_out) {
    double newb;
    *newb_out = lb;
    if (num_inf == 0) {
        newb = coeff > 0 ? surplus / coeff : slack / coeff;
        newb += ub;
    } else if (num_inf == 1 && is_posinf(ub)) {
        newb = coeff > 0 ? surplus / coeff : slack / coeff;
    } else {
        return 0;
    }
    newb = gdpo_adjust_lower(is_cont, newb);
    if (gdpo_is_lb_better(lb, ub, newb)) {
        *newb_out = newb;
        return 1;
    }
    return 0;
}

/* reference src/propagation_methods.cuh:223-276 */
void gdpo_tighten_variable(double coeff, double lhs, double rhs, double minact, double maxact,
                           int minact_inf, int maxact_inf, int is_cont, double lb, double ub,
                           int *lb_t, double *newlb, int *ub_t, double *newub) {
    const double slack = rhs - minact;
    const double surplus = lhs - maxact;
    *lb_t = 0; *newlb = lb;
    *ub_t = 0; *newub = ub;
    if (coeff > 0.0) {
        if (eps_gt(coeff * (ub - lb), rhs - minact) && !is_posinf(rhs) && !is_neginf(minact))
            *ub_t = gdpo_tighten_var_upper(coeff, slack, surplus, minact_inf, lb, ub, is_cont, newub);
        if (eps_gt(coeff * (ub - lb), maxact - lhs) && !is_neginf(lhs) && !is_posinf(maxact))
            *lb_t = gdpo_tighten_var_lower(coeff, slack, surplus, maxact_inf, lb, ub, is_cont, newlb);
    } else {
        if (eps_gt(coeff * (lb - ub), rhs - minact) && !is_posinf(rhs) && !is_neginf(minact))
            *lb_t = gdpo_tighten_var_lower(coeff, slack, surplus, minact_inf, lb, ub, is_cont, newlb);
        if (eps_gt(coeff * (lb - ub), maxact - lhs) && !is_neginf(lhs) && !is_posinf(maxact))
            *ub_t = gdpo_tighten_var_upper(coeff, slack, surplus, maxact_inf, lb, ub, is_cont, newub);
    }
}

/* reference src/propagation_methods.cuh:161-221 (left-to-right summation) */
gdpo_acts gdpo_activities(int row, const int *col, const int *row_ptr, const double *val,
                          const double *lb, const double *ub) {
    gdpo_acts a;
    double minact = 0.0, maxact = 0.0;
    int minact_inf = 0, maxact_inf = 0;
    a.maxactdelta = 0.0;
    for (int k = row_ptr[row]; k < row_ptr[row + 1]; k++) {
        const int j = col[k];
        const double coeff = val[k];
        const double l = lb[j], u = ub[j];
        const double delta = fabs(coeff) * (u - l);
        if (eps_gt(delta, a.maxactdelta)) a.maxactdelta = delta;
        const int is_min_inf = eps_gt(coeff, 0) ? is_neginf(l) : is_posinf(u);
        const int is_max_inf = eps_gt(coeff, 0) ? is_posinf(u) : is_neginf(l);
        minact_inf += is_min_inf;
        maxact_inf += is_max_inf;
        if (is_min_inf == 0) minact += coeff > 0 ? coeff * l : coeff * u;
        if (is_max_inf == 0) maxact += coeff > 0 ? coeff * u : coeff * l;
    }
    a.minact = minact; a.maxact = maxact;
    a.minact_inf = minact_inf; a.maxact_inf = maxact_inf;
    return a;
}

static inline void atomic_max_d(double *addr, double v);
static inline void atomic_min_d(double *addr, double v);

/* ---- GPU mode: the summation order of the GB300 kernels ----
 * Rows up to thread_row_max non-zeros follow the reference exactly. Longer
 * rows are summed in another order, which the GPU kernels use and the tests
 * pin bit for bit:
 *  - rows up to split_tile non-zeros are summed by a group of g lanes
 *    (gdpo_lanes_per_row): lane l sums elements l, l+g, ... in order and a
 *    shuffle tree combines the group;
 *  - longer rows are summed per warp tile of split_tile non-zeros (lane l
 *    sums elements l, l+32, ... of the tile, shuffle tree over 32 lanes),
 *    tile partials combined in tile order.
 * Every row takes the reference's row test (canConsBeTightened) with the
 * reference's sequential maxactdelta, which does not depend on how the
 * activities are summed (the kernels reach the same decision from the
 * row's FP64 maximum of |a|(ub-lb) and, where that cannot decide, the
 * sequential EPS-max itself). */
typedef struct {
    double minact, maxact;
    int minf, maxf;
} gacc;

static inline void gacc_init(gacc *s) { s->minact = 0.0; s->maxact = 0.0; s->minf = 0; s->maxf = 0; }

static inline void gacc_add(gacc *s, double coeff, double l, double u) {
    const int pos = coeff > O_EPS;
    const int lneg = l <= -O_INF, upos = u >= O_INF;
    const int min_inf = pos ? lneg : upos;
    const int max_inf = pos ? upos : lneg;
    s->minf += min_inf;
    s->maxf += max_inf;
    if (!min_inf) s->minact = s->minact + (coeff > 0 ? coeff * l : coeff * u);
    if (!max_inf) s->maxact = s->maxact + (coeff > 0 ? coeff * u : coeff * l);
}

static inline void gacc_combine(gacc *a, const gacc *b) {
    a->minact = a->minact + b->minact;
    a->maxact = a->maxact + b->maxact;
    a->minf += b->minf;
    a->maxf += b->maxf;
}

static gacc gacc_tile(int b, int e, const int *col, const double *val, const double *lb, const double *ub) {
    gacc lane[32];
    for (int l = 0; l < 32; l++) {
        gacc_init(&lane[l]);
        for (int k = b + l; k < e; k += 32) gacc_add(&lane[l], val[k], lb[col[k]], ub[col[k]]);
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int i = 0; i < off; i++) gacc_combine(&lane[i], &lane[i + off]);
    return lane[0];
}

/* Lanes per row of a SELL-g slice: rows longer than thread_row_max and at
 * most split_tile long get g = the smallest power of two >= ceil(len / 32),
 * at least 2, at most 32. */
int gdpo_lanes_per_row(int len, int thread_row_max, int tile) {
    if (len <= thread_row_max || len > tile) return 1;
    int g = 2;
    while (g < 32 && g * 32 < len) g <<= 1;
    return g;
}

/* SELL-g row: lane l of the row's group sums elements l, l+g, l+2g, ... in
 * order, then a shuffle tree (offsets g/2, ..., 1) combines the group. */
static gacc gacc_group(int b, int e, int g, const int *col, const double *val, const double *lb,
                       const double *ub) {
    gacc lane[32];
    for (int l = 0; l < g; l++) {
        gacc_init(&lane[l]);
        for (int k = b + l; k < e; k += g) gacc_add(&lane[l], val[k], lb[col[k]], ub[col[k]]);
    }
    for (int off = g / 2; off > 0; off >>= 1)
        for (int i = 0; i < off; i++) gacc_combine(&lane[i], &lane[i + off]);
    return lane[0];
}

static gacc gpu_row_acts(int row, const int *col, const int *row_ptr, const double *val, const double *lb,
                         const double *ub, int thread_row_max, int tile) {
    const int b0 = row_ptr[row], e0 = row_ptr[row + 1];
    gacc a;
    if (e0 - b0 <= thread_row_max) {
        gacc_init(&a);
        for (int k = b0; k < e0; k++) gacc_add(&a, val[k], lb[col[k]], ub[col[k]]);
        return a;
    }
    if (e0 - b0 <= tile) return gacc_group(b0, e0, gdpo_lanes_per_row(e0 - b0, thread_row_max, tile), col, val, lb, ub);
    a = gacc_tile(b0, b0 + tile < e0 ? b0 + tile : e0, col, val, lb, ub);
    for (int b = b0 + tile; b < e0; b += tile) {
        const gacc t = gacc_tile(b, b + tile < e0 ? b + tile : e0, col, val, lb, ub);
        gacc_combine(&a, &t);
    }
    return a;
}

/* The reference's maxactdelta of a row: the sequential EPS-max of
 * |a|(ub-lb) in row order (src/propagation_methods.cuh:188-190). */
static double seq_maxactdelta(int row, const int *col, const int *row_ptr, const double *val, const double *lb,
                              const double *ub) {
    double m = 0.0;
    for (int k = row_ptr[row]; k < row_ptr[row + 1]; k++) {
        const double d = fabs(val[k]) * (ub[col[k]] - lb[col[k]]);
        if (eps_gt(d, m)) m = d;
    }
    return m;
}

static int jacobi_row(int row, const int *col, const int *row_ptr, const double *val,
                      const double *lhs, const double *rhs, const double *lb, const double *ub,
                      const int *vartype, double *lb_out, double *ub_out,
                      unsigned char *var_changed, int *go, int *infeas);

/* Rows up to thread_row_max non-zeros follow the reference exactly
 * (jacobi_row). Longer rows: the kernels' summation order, the reference's
 * row test and candidates. */
static int jacobi_row_gpu(int row, const int *col, const int *row_ptr, const double *val, const double *lhs,
                          const double *rhs, const double *lb, const double *ub, const int *vartype,
                          double *lb_out, double *ub_out, unsigned char *var_changed, int thread_row_max,
                          int tile, int *go, int *infeas) {
    if (row_ptr[row + 1] - row_ptr[row] <= thread_row_max)
        return jacobi_row(row, col, row_ptr, val, lhs, rhs, lb, ub, vartype, lb_out, ub_out, var_changed, go,
                          infeas);
    const gacc a = gpu_row_acts(row, col, row_ptr, val, lb, ub, thread_row_max, tile);
    *infeas = gdpo_row_infeasible(a.minact, a.maxact, a.minf, a.maxf, lhs[row], rhs[row]);
    *go = gdpo_can_cons_be_tightened(a.minact, a.maxact, a.minf, a.maxf, lhs[row], rhs[row],
                                     seq_maxactdelta(row, col, row_ptr, val, lb, ub));
    if (!*go) return 0;
    int any = 0;
    for (int k = row_ptr[row]; k < row_ptr[row + 1]; k++) {
        const int j = col[k];
        int lt, ut;
        double nl, nu;
        gdpo_tighten_variable(val[k], lhs[row], rhs[row], a.minact, a.maxact, a.minf, a.maxf, vartype[j] == 3,
                              lb[j], ub[j], &lt, &nl, &ut, &nu);
        if (lt) atomic_max_d(&lb_out[j], nl);
        if (ut) atomic_min_d(&ub_out[j], nu);
        if (lt || ut) {
            any = 1;
            if (var_changed) __atomic_store_n(&var_changed[j], (unsigned char)1, __ATOMIC_RELAXED);
        }
    }
    return any;
}

/* Infeasibility rule of this project (the reference detects none): bounds
 * crossing by more than a relative feasibility tolerance. */
int gdpo_var_infeasible(double lb, double ub) {
    double s = fabs(lb) > fabs(ub) ? fabs(lb) : fabs(ub);
    if (s < 1.0) s = 1.0;
    return (lb - ub) > O_FEASTOL * s;
}

/* --- order-independent candidate application (max for lb, min for ub) --- */
static inline void atomic_max_d(double *addr, double v) {
    uint64_t *p = (uint64_t *)addr;
    uint64_t old = __atomic_load_n(p, __ATOMIC_RELAXED);
    for (;;) {
        double od;
        memcpy(&od, &old, 8);
        if (!(v > od)) return;
        uint64_t nv;
        memcpy(&nv, &v, 8);
        if (__atomic_compare_exchange_n(p, &old, nv, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
    }
}
static inline void atomic_min_d(double *addr, double v) {
    uint64_t *p = (uint64_t *)addr;
    uint64_t old = __atomic_load_n(p, __ATOMIC_RELAXED);
    for (;;) {
        double od;
        memcpy(&od, &old, 8);
        if (!(v < od)) return;
        uint64_t nv;
        memcpy(&nv, &v, 8);
        if (__atomic_compare_exchange_n(p, &old, nv, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
    }
}

/* One Jacobi row: reference src/propagators/OMP_propagator.h:58-131, with the
 * locked "apply if better" replaced by max/min of the gated candidates. */
static int jacobi_row(int row, const int *col, const int *row_ptr, const double *val,
                      const double *lhs, const double *rhs, const double *lb, const double *ub,
                      const int *vartype, double *lb_out, double *ub_out,
                      unsigned char *var_changed, int *go, int *infeas) {
    const gdpo_acts a = gdpo_activities(row, col, row_ptr, val, lb, ub);
    int any = 0;
    *infeas = gdpo_row_infeasible(a.minact, a.maxact, a.minact_inf, a.maxact_inf, lhs[row], rhs[row]);
    *go = gdpo_can_cons_be_tightened(a.minact, a.maxact, a.minact_inf, a.maxact_inf, lhs[row], rhs[row],
                                     a.maxactdelta);
    if (!*go) return 0;
    for (int k = row_ptr[row]; k < row_ptr[row + 1]; k++) {
        const int j = col[k];
        int lt, ut;
        double nl, nu;
        gdpo_tighten_variable(val[k], lhs[row], rhs[row], a.minact, a.maxact, a.minact_inf,
                              a.maxact_inf, vartype[j] == 3, lb[j], ub[j], &lt, &nl, &ut, &nu);
        if (lt) atomic_max_d(&lb_out[j], nl);
        if (ut) atomic_min_d(&ub_out[j], nu);
        if (lt || ut) {
            any = 1;
            if (var_changed) __atomic_store_n(&var_changed[j], (unsigned char)1, __ATOMIC_RELAXED);
        }
    }
    return any;
}

int gdpo_jacobi_round(int m, int n, const int *col, const int *row_ptr, const double *val,
                      const double *lhs, const double *rhs, const double *lb, const double *ub,
                      const int *vartype, const unsigned char *mark, double *lb_out,
                      double *ub_out, unsigned char *tight_row, int nthreads) {
    int change = 0;
    (void)n;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads > 0 ? nthreads : 1) reduction(| : change)
#endif
    for (int i = 0; i < m; i++) {
        if (mark && !mark[i]) continue;
        int go, infeas;
        const int t = jacobi_row(i, col, row_ptr, val, lhs, rhs, lb, ub, vartype, lb_out, ub_out, NULL, &go,
                                 &infeas);
        if (t && tight_row) tight_row[i] = 1;
        change |= t;
    }
    return change;
}

/* CSC of the sparsity pattern (row indices per column), used for marking:
 * the reference builds it with cuSPARSE (src/kernels/util_kernels.cuh:92-152). */
static void build_csc(int m, int n, int nnz, const int *col, const int *row_ptr, int *col_ptr,
                      int *row_idx) {
    memset(col_ptr, 0, sizeof(int) * (size_t)(n + 1));
    for (int k = 0; k < nnz; k++) col_ptr[col[k] + 1]++;
    for (int j = 0; j < n; j++) col_ptr[j + 1] += col_ptr[j];
    int *fill = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    memcpy(fill, col_ptr, sizeof(int) * (size_t)n);
    for (int i = 0; i < m; i++)
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) row_idx[fill[col[k]]++] = i;
    free(fill);
}

static int check_input(int m, int n, int nnz, const int *col, const int *row_ptr) {
    if (m < 0 || n < 0 || nnz < 0) return -1;
    if (row_ptr[0] != 0 || row_ptr[m] != nnz) return -2;
    for (int i = 0; i < m; i++)
        if (row_ptr[i + 1] < row_ptr[i]) return -3;
    for (int k = 0; k < nnz; k++)
        if (col[k] < 0 || col[k] >= n) return -4;
    return 0;
}

/* Fixpoint loop: reference src/propagators/sequential_propagator.h:241-278
 * (SEQUENTIAL) and src/propagators/OMP_propagator.h:168-211 (JACOBI), with a
 * configurable round cap and the infeasibility rule checked after each round. */
int gdpo_propagate(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                   const double *lhs, const double *rhs, double *lb, double *ub,
                   const int *vartype, int schedule, int max_rounds, int nthreads,
                   gdpo_result *res) {
    return gdpo_propagate_ex(m, n, nnz, col, row_ptr, val, lhs, rhs, lb, ub, vartype, schedule,
                             max_rounds, nthreads, 0, 0, res);
}

int gdpo_propagate_ex(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                      const double *lhs, const double *rhs, double *lb, double *ub,
                      const int *vartype, int schedule, int max_rounds, int nthreads,
                      int split_len, int split_tile, gdpo_result *res) {
    gdpo_result r;
    const int gpu_mode = split_tile > 0;
    memset(&r, 0, sizeof(r));
    r.infeasible_var = -1;
    r.infeasible_row = -1;
    if (max_rounds <= 0) max_rounds = O_MAX_ROUNDS;
    if (m == 0 || n == 0 || nnz == 0) {
        r.converged = 1;
        if (res) *res = r;
        return 0;
    }
    const int rc = check_input(m, n, nnz, col, row_ptr);
    if (rc) return rc;

    for (int j = 0; j < n; j++)
        if (gdpo_var_infeasible(lb[j], ub[j])) {
            r.infeasible = 1;
            r.infeasible_var = j;
            r.converged = 1;
            if (res) *res = r;
            return 0;
        }

    int *col_ptr = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    int *row_idx = (int *)malloc(sizeof(int) * (size_t)nnz);
    build_csc(m, n, nnz, col, row_ptr, col_ptr, row_idx);
    unsigned char *mark = (unsigned char *)malloc((size_t)m);
    unsigned char *var_changed = (unsigned char *)calloc((size_t)n, 1);
    double *lb_snap = (double *)malloc(sizeof(double) * (size_t)n);
    double *ub_snap = (double *)malloc(sizeof(double) * (size_t)n);
    memset(mark, 1, (size_t)m); /* every row is marked in round 1 */

    int change = 1;
    while (r.rounds < max_rounds && change && !r.infeasible) {
        r.rounds++;
        change = 0;
        long long rows = 0, nz = 0, cands = 0, go_rows = 0;
        int inf_row = INT_MAX; /* smallest row found infeasible in this round */
        for (int i = 0; i < m; i++)
            if (mark[i]) { rows++; nz += row_ptr[i + 1] - row_ptr[i]; }
        if (schedule == GDPO_SCHED_SEQUENTIAL) {
            /* reference src/propagators/sequential_propagator.h:46-121 */
            for (int i = 0; i < m; i++) {
                if (!mark[i]) continue;
                const gdpo_acts a = gdpo_activities(i, col, row_ptr, val, lb, ub);
                if (inf_row == INT_MAX &&
                    gdpo_row_infeasible(a.minact, a.maxact, a.minact_inf, a.maxact_inf, lhs[i], rhs[i]))
                    inf_row = i;
                if (!gdpo_can_cons_be_tightened(a.minact, a.maxact, a.minact_inf, a.maxact_inf,
                                                lhs[i], rhs[i], a.maxactdelta))
                    continue;
                for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
                    const int j = col[k];
                    int lt, ut;
                    double nl, nu;
                    gdpo_tighten_variable(val[k], lhs[i], rhs[i], a.minact, a.maxact,
                                          a.minact_inf, a.maxact_inf, vartype[j] == 3, lb[j],
                                          ub[j], &lt, &nl, &ut, &nu);
                    if (lt) lb[j] = nl;
                    if (ut) ub[j] = nu;
                    if (lt || ut) { change = 1; var_changed[j] = 1; cands += lt + ut; }
                }
            }
        } else {
            memcpy(lb_snap, lb, sizeof(double) * (size_t)n);
            memcpy(ub_snap, ub, sizeof(double) * (size_t)n);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads > 0 ? nthreads : 1) \
        reduction(| : change) reduction(+ : go_rows) reduction(min : inf_row)
#endif
            for (int i = 0; i < m; i++) {
                if (!mark[i]) continue;
                int go = 0, infeas = 0;
                if (gpu_mode) {
                    change |= jacobi_row_gpu(i, col, row_ptr, val, lhs, rhs, lb_snap, ub_snap, vartype, lb,
                                             ub, var_changed, split_len, split_tile, &go, &infeas);
                    if (go && row_ptr[i + 1] - row_ptr[i] <= split_tile) go_rows++;
                } else {
                    change |= jacobi_row(i, col, row_ptr, val, lhs, rhs, lb_snap, ub_snap, vartype, lb,
                                         ub, var_changed, &go, &infeas);
                }
                if (infeas && i < inf_row) inf_row = i;
            }
        }
        /* marking for the next round: reference src/propagation_methods.cu:3-13 */
        memset(mark, 0, (size_t)m);
        for (int j = 0; j < n; j++) {
            if (!var_changed[j]) continue;
            var_changed[j] = 0;
            if (schedule != GDPO_SCHED_SEQUENTIAL) cands++;
            for (int k = col_ptr[j]; k < col_ptr[j + 1]; k++) mark[row_idx[k]] = 1;
            if (r.infeasible_var < 0 && gdpo_var_infeasible(lb[j], ub[j])) {
                r.infeasible = 1;
                r.infeasible_var = j;
            }
        }
        if (inf_row != INT_MAX) {
            r.infeasible = 1;
            r.infeasible_row = inf_row;
        }
        r.rows_processed += rows;
        r.nnz_processed += nz;
        r.rows_go += go_rows;
        r.candidates += cands;
    }
    r.converged = !change || r.infeasible;

    free(col_ptr); free(row_idx); free(mark); free(var_changed); free(lb_snap); free(ub_snap);
    if (res) *res = r;
    return 0;
}

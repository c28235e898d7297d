/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Drives the reference's OWN round functions, compiled from the reference
 * sources by oracle/Makefile into oracle/_ref/libgdpref.so (in the build
 * container, where the reference sources exist). Used to pin the oracle
 * restatement (oracle/gdp_oracle.c) and as the reference CPU baseline.
 *
 * The reference's fixed-cap drivers (sequentialPropagate, fullOMPPropagate)
 * are not called: this harness mirrors their loops
 * (src/propagators/sequential_propagator.h:241-278,
 *  src/propagators/OMP_propagator.h:168-211) around the reference's
 * sequentialPropagationRound<double> / OMPPropagationRound<double> with a
 * configurable round cap, the project's infeasibility rules after each round
 * (untimed: variable crossing, and the row rule on the activities the round
 * function left in minacts/maxacts for every row it processed) and wall-clock
 * timing of the round calls only, which is where the reference places its own
 * timers.
 */
#include "propagators/sequential_propagator.h"
#include "propagators/OMP_propagator.h"

#include <chrono>
#include <vector>

namespace {

bool var_infeasible(double lb, double ub) {
    double s = std::fabs(lb) > std::fabs(ub) ? std::fabs(lb) : std::fabs(ub);
    if (s < 1.0) s = 1.0;
    return (lb - ub) > 1e-6 * s;
}

/* The row rule: the reference's isConsInfeasible on a side with a finite
 * constraint side and no infinite contribution, relative tolerance 1e-6. */
bool row_infeasible(double minact, double maxact, int minf, int maxf, double lhs, double rhs) {
    if (minf == 0 && !ISPOSINF(rhs)) {
        double s = std::fabs(minact) > std::fabs(rhs) ? std::fabs(minact) : std::fabs(rhs);
        if (s < 1.0) s = 1.0;
        if (minact - rhs > 1e-6 * s) return true;
    }
    if (maxf == 0 && !ISNEGINF(lhs)) {
        double s = std::fabs(maxact) > std::fabs(lhs) ? std::fabs(maxact) : std::fabs(lhs);
        if (s < 1.0) s = 1.0;
        if (lhs - maxact > 1e-6 * s) return true;
    }
    return false;
}

/* CSC pattern by counting sort (the reference uses cuSPARSE for this). */
void build_csc(int m, int n, int nnz, const int *col, const int *row_ptr,
               std::vector<int> &col_ptr, std::vector<int> &row_idx) {
    col_ptr.assign(n + 1, 0);
    row_idx.assign(nnz > 0 ? nnz : 1, 0);
    for (int k = 0; k < nnz; k++) col_ptr[col[k] + 1]++;
    for (int j = 0; j < n; j++) col_ptr[j + 1] += col_ptr[j];
    std::vector<int> fill(col_ptr.begin(), col_ptr.end() - 1);
    for (int i = 0; i < m; i++)
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) row_idx[fill[col[k]]++] = i;
}

}  // namespace

extern "C" {

/* schedule 0: cpu_omp round function (SHARED_MEM_THREADS OpenMP threads);
 * schedule 1: cpu_seq round function. Returns 0 on success. */
int gdpref_propagate(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                     const double *lhs, const double *rhs, double *lb, double *ub,
                     const int *vartype, int schedule, int max_rounds, int *rounds_out,
                     int *infeasible_out, int *converged_out, double *seconds_out) {
    *rounds_out = 0;
    *infeasible_out = 0;
    *converged_out = 1;
    *seconds_out = 0.0;
    if (m == 0 || n == 0 || nnz == 0) return 0;
    if (max_rounds <= 0) max_rounds = MAX_NUM_ROUNDS;
    for (int j = 0; j < n; j++)
        if (var_infeasible(lb[j], ub[j])) { *infeasible_out = 1; return 0; }

    std::vector<int> csc_col_ptrs, csc_row_indices;
    build_csc(m, n, nnz, col, row_ptr, csc_col_ptrs, csc_row_indices);
    const GDP_VARTYPE *vt = reinterpret_cast<const GDP_VARTYPE *>(vartype);

    std::vector<double> minacts(m), maxacts(m), maxactdeltas(m), lbs_local(n), ubs_local(n);
    std::vector<int> minacts_inf(m), maxacts_inf(m), consmarked(m, 1), consmarked_next(m, 0);
    std::vector<omp_lock_t> locks(schedule == 0 ? n : 0);
    for (auto &l : locks) omp_init_lock(&l);

    bool change_found = true;
    bool infeasible = false;
    int round = 0;
    double seconds = 0.0;
    std::vector<double> lb_before(n), ub_before(n);
    std::vector<int> marked_before(m);
    while (round < max_rounds && change_found && !infeasible) {
        round++;
        std::copy(lb, lb + n, lb_before.begin());
        std::copy(ub, ub + n, ub_before.begin());
        std::copy(consmarked.begin(), consmarked.end(), marked_before.begin());
        auto t0 = std::chrono::steady_clock::now();
        if (schedule == 0) {
            change_found = OMPPropagationRound<double>(
                    m, n, col, row_ptr, csc_col_ptrs.data(), csc_row_indices.data(), val, lhs, rhs,
                    lb, ub, lbs_local.data(), ubs_local.data(), vt, minacts.data(), maxacts.data(),
                    minacts_inf.data(), maxacts_inf.data(), maxactdeltas.data(), consmarked.data(),
                    locks.data(), consmarked_next.data(), round);
        } else {
            change_found = sequentialPropagationRound<double>(
                    m, n, col, row_ptr, csc_col_ptrs.data(), csc_row_indices.data(), val, lhs, rhs,
                    lb, ub, vt, minacts.data(), maxacts.data(), minacts_inf.data(),
                    maxacts_inf.data(), maxactdeltas.data(), consmarked.data(),
                    consmarked_next.data(), RECOMPUTE_ACTS_TRUE);
        }
        seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (int j = 0; j < n && !infeasible; j++)
            if ((lb[j] != lb_before[j] || ub[j] != ub_before[j]) && var_infeasible(lb[j], ub[j]))
                infeasible = true;
        for (int i = 0; i < m && !infeasible; i++)
            if (marked_before[i] &&
                row_infeasible(minacts[i], maxacts[i], minacts_inf[i], maxacts_inf[i], lhs[i], rhs[i]))
                infeasible = true;
    }
    for (auto &l : locks) omp_destroy_lock(&l);
    *rounds_out = round;
    *infeasible_out = infeasible ? 1 : 0;
    *converged_out = (!change_found || infeasible) ? 1 : 0;
    *seconds_out = seconds;
    return 0;
}

/* The reference's computeActivities for one row (known-answer checks). */
void gdpref_activities(int row, const int *col, const int *row_ptr, const double *val,
                       const double *lb, const double *ub, double *minact, double *maxact,
                       double *maxactdelta, int *minact_inf, int *maxact_inf) {
    ActivitiesTuple a = computeActivities<double>(row, col, row_ptr, val, ub, lb);
    *minact = a.minact;
    *maxact = a.maxact;
    *maxactdelta = a.maxactdelta;
    *minact_inf = a.minact_inf;
    *maxact_inf = a.maxact_inf;
}

}  // extern "C"

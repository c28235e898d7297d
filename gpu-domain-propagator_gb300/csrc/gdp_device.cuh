// gdp_device.cuh -- FP64 propagation math on the device (sm_103a).
//
// Every expression rounds exactly like the reference's host code
// (src/propagation_methods.cuh): explicit round-to-nearest intrinsics keep
// nvcc from contracting a*b+c into an FMA, and divisions are IEEE div.rn.
// Comparisons against the +-GDP_INF constants use the plain ordered form,
// which is exactly equivalent to the reference's EPS form for every double
// (including +-inf and NaN):
//   EPSGE(x, 1e20) == (x >= 1e20) and EPSLE(x, -1e20) == (x <= -1e20),
// because every double within 5e19..2e20 of 1e20 differs from it by a multiple
// of ulp(1e20) = 16384 (Sterbenz), and everything else differs by >= 5e19.
#pragma once

#include <cstdint>

namespace gdp {

constexpr double kInf = 1e20;
constexpr double kEps = 1e-9;
constexpr double kFeasTol = 1e-6;

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// reference src/def.h:68-79
__device__ __forceinline__ bool eps_gt(double x, double y) { return dsub(x, y) > kEps; }
__device__ __forceinline__ bool eps_lt(double x, double y) { return dsub(x, y) < -kEps; }
__device__ __forceinline__ bool eps_le(double x, double y) { return dsub(x, y) <= kEps; }
__device__ __forceinline__ bool is_posinf(double x) { return x >= kInf; }
__device__ __forceinline__ bool is_neginf(double x) { return x <= -kInf; }
__device__ __forceinline__ double eps_floor(double x) { return floor(dadd(x, kEps)); }
__device__ __forceinline__ double eps_ceil(double x) { return ceil(dsub(x, kEps)); }

// Row statistics (reference ActivitiesTuple, src/propagation_methods.cuh:10-17).
struct RowActs {
    double minact, maxact, maxactdelta;
    int minact_inf, maxact_inf;
};

// One term of computeActivities (src/propagation_methods.cuh:188-214), added
// to the running left-to-right state.
__device__ __forceinline__ void acts_add(RowActs &a, double coeff, double lb, double ub) {
    const double delta = dmul(fabs(coeff), dsub(ub, lb));
    if (eps_gt(delta, a.maxactdelta)) a.maxactdelta = delta;
    const bool pos = coeff > kEps;  // EPSGT(coeff, 0): coeff - 0 is exact
    const bool min_inf = pos ? is_neginf(lb) : is_posinf(ub);
    const bool max_inf = pos ? is_posinf(ub) : is_neginf(lb);
    a.minact_inf += min_inf;
    a.maxact_inf += max_inf;
    const bool gt0 = coeff > 0.0;
    if (!min_inf) a.minact = dadd(a.minact, dmul(coeff, gt0 ? lb : ub));
    if (!max_inf) a.maxact = dadd(a.maxact, dmul(coeff, gt0 ? ub : lb));
}

__device__ __forceinline__ void acts_init(RowActs &a) {
    a.minact = 0.0; a.maxact = 0.0; a.maxactdelta = 0.0; a.minact_inf = 0; a.maxact_inf = 0;
}

// reference canConsBeTightened, src/propagation_methods.cuh:136-154
__device__ __forceinline__ bool can_cons_be_tightened(const RowActs &a, double lhs, double rhs) {
    if (a.minact_inf > 1 && a.maxact_inf > 1) return false;
    if (a.maxactdelta < kInf) {  // EPSLT(maxactdelta, GDP_INF)
        const double s = dsub(rhs, a.minact), t = dsub(a.maxact, lhs);
        return !eps_le(a.maxactdelta, (t < s) ? t : s);  // std::min(s, t)
    }
    return true;
}

// Per-row constants of tightenVariable (src/propagation_methods.cuh:223-276).
struct RowCand {
    double slack, surplus, neg_surplus;  // rhs - minact, lhs - maxact, maxact - lhs
    int minact_inf, maxact_inf;
    bool rhs_side_ok;  // !ISPOSINF(rhs) && !ISNEGINF(minact)
    bool lhs_side_ok;  // !ISNEGINF(lhs) && !ISPOSINF(maxact)
};

__device__ __forceinline__ RowCand row_cand(const RowActs &a, double lhs, double rhs) {
    RowCand c;
    c.slack = dsub(rhs, a.minact);
    c.surplus = dsub(lhs, a.maxact);
    c.neg_surplus = dsub(a.maxact, lhs);
    c.minact_inf = a.minact_inf;
    c.maxact_inf = a.maxact_inf;
    c.rhs_side_ok = !is_posinf(rhs) && !is_neginf(a.minact);
    c.lhs_side_ok = !is_neginf(lhs) && !is_posinf(a.maxact);
    return c;
}

// tightenVarUpperBound, src/propagation_methods.cuh:78-106
__device__ __forceinline__ bool tighten_upper(double coeff, const RowCand &c, int num_inf, double lb,
                                              double ub, bool is_cont, double &newb) {
    if (!(num_inf == 0 || (num_inf == 1 && is_neginf(lb)))) return false;
    double nb = ddiv(coeff > 0 ? c.slack : c.surplus, coeff);
    if (num_inf == 0) nb = dadd(nb, lb);
    if (!is_cont) nb = eps_floor(nb);
    if (eps_lt(nb, ub)) { newb = nb; return true; }
    return false;
}

// tightenVarLowerBound, src/propagation_methods.cuh:108-134
__device__ __forceinline__ bool tighten_lower(double coeff, const RowCand &c, int num_inf, double lb,
                                              double ub, bool is_cont, double &newb) {
    if (!(num_inf == 0 || (num_inf == 1 && is_posinf(ub)))) return false;
    double nb = ddiv(coeff > 0 ? c.surplus : c.slack, coeff);
    if (num_inf == 0) nb = dadd(nb, ub);
    if (!is_cont) nb = eps_ceil(nb);
    if (eps_gt(nb, lb)) { newb = nb; return true; }
    return false;
}

// tightenVariable, src/propagation_methods.cuh:223-276. coeff*(ub-lb) for
// coeff > 0 and coeff*(lb-ub) otherwise both equal |coeff|*(ub-lb) bit for bit
// (round-to-nearest is sign-symmetric), so one product serves both branches.
__device__ __forceinline__ void tighten_variable(double coeff, const RowCand &c, bool is_cont, double lb,
                                                 double ub, bool &lb_t, double &newlb, bool &ub_t,
                                                 double &newub) {
    lb_t = false;
    ub_t = false;
    const double d = dmul(fabs(coeff), dsub(ub, lb));
    const bool rhs_side = c.rhs_side_ok && eps_gt(d, c.slack);
    const bool lhs_side = c.lhs_side_ok && eps_gt(d, c.neg_surplus);
    if (coeff > 0.0) {
        if (rhs_side) ub_t = tighten_upper(coeff, c, c.minact_inf, lb, ub, is_cont, newub);
        if (lhs_side) lb_t = tighten_lower(coeff, c, c.maxact_inf, lb, ub, is_cont, newlb);
    } else {
        if (rhs_side) lb_t = tighten_lower(coeff, c, c.minact_inf, lb, ub, is_cont, newlb);
        if (lhs_side) ub_t = tighten_upper(coeff, c, c.maxact_inf, lb, ub, is_cont, newub);
    }
}

// FP64 max / min as one integer atomic each: for sign bit 0 the bit pattern
// orders like a signed integer; for sign bit 1 it orders in reverse as an
// unsigned integer. No CAS loop, no return value (RED.MAX / RED.MIN).
__device__ __forceinline__ void atomic_max_f64(double *addr, double v) {
    const long long b = __double_as_longlong(v);
    if (b >= 0) atomicMax(reinterpret_cast<long long *>(addr), b);
    else atomicMin(reinterpret_cast<unsigned long long *>(addr), static_cast<unsigned long long>(b));
}
__device__ __forceinline__ void atomic_min_f64(double *addr, double v) {
    const long long b = __double_as_longlong(v);
    if (b >= 0) atomicMin(reinterpret_cast<long long *>(addr), b);
    else atomicMax(reinterpret_cast<unsigned long long *>(addr), static_cast<unsigned long long>(b));
}

// The project's infeasibility rule (the reference detects none).
__device__ __forceinline__ bool var_infeasible(double lb, double ub) {
    double s = fmax(fabs(lb), fabs(ub));
    if (s < 1.0) s = 1.0;
    return dsub(lb, ub) > dmul(kFeasTol, s);
}

}  // namespace gdp

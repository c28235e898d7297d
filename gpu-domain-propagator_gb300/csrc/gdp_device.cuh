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

// ---- integer-domain forms (no FP64 pipe) ----------------------------------
// Exact for every non-NaN double: a double's bit pattern orders like a signed
// integer when the sign bit is 0, and in reverse as an unsigned integer when
// it is 1.
constexpr long long kBitsEps = 0x3E112E0BE826D695LL;          // 1e-9
constexpr long long kBitsPosInf = 0x4415AF1D78B58C40LL;       // 1e20
constexpr unsigned long long kBitsNegInf = 0xC415AF1D78B58C40ULL;  // -1e20

__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
// x > 1e-9 (the reference's EPSGT(x, 0))
__device__ __forceinline__ bool gt_eps_bits(long long b) { return b > kBitsEps; }
// x > 0
__device__ __forceinline__ bool gt0_bits(long long b) { return b > 0; }
// x <= -1e20 (ISNEGINF)
__device__ __forceinline__ bool neginf_bits(long long b) { return (unsigned long long)b >= kBitsNegInf; }
// x >= 1e20 (ISPOSINF)
__device__ __forceinline__ bool posinf_bits(long long b) { return b >= kBitsPosInf; }
// key(x) < key(y) iff x < y for non-NaN doubles (NaN keys sort above +inf)
__device__ __forceinline__ long long order_key(long long b) {
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
// EPSGT(x, y) with the FP64 subtraction only when x > y.
__device__ __forceinline__ bool eps_gt_fast(double x, double y) {
    return order_key(dbits(x)) > order_key(dbits(y)) && eps_gt(x, y);
}

// Outward rounding of a double to float by integer arithmetic.
__device__ __forceinline__ float f32_mag(unsigned long long mag, bool up) {
    const int e = (int)(mag >> 52);
    if (e == 2047) return (mag & 0xFFFFFFFFFFFFFULL) ? __uint_as_float(0x7FC00000u) : __uint_as_float(0x7F800000u);
    const int fe = e - 1023 + 127;
    if (fe >= 255) return up ? __uint_as_float(0x7F800000u) : __uint_as_float(0x7F7FFFFFu);
    if (fe <= 0) return (up && mag) ? __uint_as_float(0x00800000u) : 0.0f;
    const unsigned long long man = mag & 0xFFFFFFFFFFFFFULL;
    unsigned fb = ((unsigned)fe << 23) | (unsigned)(man >> 29);
    if (up && (man & 0x1FFFFFFFULL)) fb += 1u;
    return __uint_as_float(fb);
}
__device__ __forceinline__ float f32_up(long long b) {
    const unsigned long long mag = (unsigned long long)b & 0x7FFFFFFFFFFFFFFFULL;
    return b < 0 ? -f32_mag(mag, false) : f32_mag(mag, true);
}
__device__ __forceinline__ float f32_dn(long long b) {
    const unsigned long long mag = (unsigned long long)b & 0x7FFFFFFFFFFFFFFFULL;
    return b < 0 ? -f32_mag(mag, true) : f32_mag(mag, false);
}
constexpr float kUMargin = 1.00000095367431640625f;  // 1 + 2^-20

// Sign-aware FP32 enclosure lo <= |a| (ub - lb) <= hi of one element, each end
// widened by a relative 2^-20 (covers the round-to-nearest float operations).
// NaN (e.g. inf - inf) makes every comparison inconclusive, which sends the
// element to the exact FP64 path.
struct DeltaBox {
    float lo, hi;
};
__device__ __forceinline__ float widen_up(float x) { return __fadd_rn(x, fabsf(x) * 9.5367431640625e-7f); }
__device__ __forceinline__ float widen_dn(float x) { return __fsub_rn(x, fabsf(x) * 9.5367431640625e-7f); }
__device__ __forceinline__ DeltaBox delta_box(long long ab, long long lbb, long long ubb) {
    const unsigned long long am = (unsigned long long)ab & 0x7FFFFFFFFFFFFFFFULL;
    const float a_up = f32_mag(am, true), a_dn = f32_mag(am, false);
    const float dh = __fsub_rn(f32_up(ubb), f32_dn(lbb));  // >= ub - lb (up to rounding)
    const float dl = __fsub_rn(f32_dn(ubb), f32_up(lbb));  // <= ub - lb (up to rounding)
    DeltaBox b;
    b.hi = widen_up(__fmul_rn(dh >= 0.0f ? a_up : a_dn, dh));
    b.lo = widen_dn(__fmul_rn(dl >= 0.0f ? a_dn : a_up, dl));
    return b;
}

// Activity accumulator: the reference's computeActivities terms with integer
// classification (no FP64 compares), plus the first maximum of the FP64
// |a| (ub - lb) over the elements seen: km is its order key (order_key of its
// bit pattern; the maximum is never negative, so km is its bit pattern), p its
// element index within the row. The virtual element 0.0 at index -1 stands for
// the initial value of the reference's maxactdelta, so km >= 0 always.
struct Acc {
    double minact, maxact;
    int minf, maxf;
    long long km;
    int p;
};
__device__ __forceinline__ void acc_init(Acc &s) {
    s.minact = 0.0; s.maxact = 0.0; s.minf = 0; s.maxf = 0; s.km = 0; s.p = -1;
}
// Order key of +inf: keys above it are NaN, which the reference's EPSGT never
// takes as a new maximum.
constexpr long long kKeyPosInf = 0x7FF0000000000000LL;
// Element k with d = fl(|a| fl(ub - lb)) (the reference's maxactdelta term):
// elements are visited in increasing k per accumulator, so a strict compare
// keeps the first index of the maximum.
__device__ __forceinline__ void acc_add_delta(Acc &s, double d, int k) {
    const long long kd = order_key(dbits(d));
    if (kd > s.km && kd <= kKeyPosInf) {
        s.km = kd;
        s.p = k;
    }
}
// Combines first maxima: the larger, of equal ones the earlier element.
__device__ __forceinline__ void acc_take_max(Acc &s, long long km, int p) {
    if (km > s.km || (km == s.km && p < s.p)) {
        s.km = km;
        s.p = p;
    }
}
__device__ __forceinline__ double acc_max(const Acc &s) { return __longlong_as_double(s.km); }
// The activity terms and infinity counts of one element.
__device__ __forceinline__ void acc_add_terms(Acc &s, double a, double lb, double ub) {
    const long long ab = dbits(a), lbb = dbits(lb), ubb = dbits(ub);
    const bool pos = gt_eps_bits(ab);
    const bool lneg = neginf_bits(lbb), upos = posinf_bits(ubb);
    const bool min_inf = pos ? lneg : upos;
    const bool max_inf = pos ? upos : lneg;
    s.minf += min_inf;
    s.maxf += max_inf;
    const bool gt0 = gt0_bits(ab);
    if (!min_inf) s.minact = dadd(s.minact, dmul(a, gt0 ? lb : ub));
    if (!max_inf) s.maxact = dadd(s.maxact, dmul(a, gt0 ? ub : lb));
}
__device__ __forceinline__ void acc_combine(Acc &a, const Acc &b) {
    a.minact = dadd(a.minact, b.minact);
    a.maxact = dadd(a.maxact, b.maxact);
    a.minf += b.minf;
    a.maxf += b.maxf;
    acc_take_max(a, b.km, b.p);
}

// min(rhs - minact, maxact - lhs) as std::min(s, t) in canConsBeTightened.
__device__ __forceinline__ double row_min_slack(double minact, double maxact, double lhs, double rhs) {
    const double s = dsub(rhs, minact), t = dsub(maxact, lhs);
    return (t < s) ? t : s;
}
// The reference's decision from its sequential maxactdelta (canConsBeTightened).
__device__ __forceinline__ bool reference_row_go(int minf, int maxf, double maxactdelta, double mn) {
    if (minf > 1 && maxf > 1) return false;
    if (maxactdelta < kInf) return !eps_le(maxactdelta, mn);
    return true;
}

// The reference's row test (canConsBeTightened, src/propagation_methods.cuh:
// 136-154) from the row's FP64 maximum M of |a| (ub - lb) (with the leading
// 0.0) instead of its sequential EPS-max m (computeActivities :188-190, where
// an element replaces m only when it exceeds m by more than EPS).
// Let p be the first index of M. After element p, m = M unless
// fl(M - m_before) <= EPS; later elements never replace m. Hence m <= M, and
// m >= M - EPS - ulp(EPS)/2 (Sterbenz makes M - m_before exact unless both are
// below 2 EPS). m >= 1e20 exactly when M >= 1e20 (doubles near 1e20 are 16384
// apart). So, with v = fl(M - mn):
//   v <= EPS                      -> fl(m - mn) <= v: the reference skips;
//   v > kGoClear (2.00001e-9)     -> m - mn > 1.00001e-9: it processes the row;
//   in between                    -> only m itself decides (seq_eps_max).
// Returns 0 (skip), 1 (process) or 2 (undecided: compute m).
constexpr double kGoClear = 2.00001e-9;
__device__ __forceinline__ int row_go_from_max(int minf, int maxf, double M, double mn) {
    if (minf > 1 && maxf > 1) return 0;
    if (M >= kInf) return 1;
    const double v = dsub(M, mn);
    if (v <= kEps) return 0;
    return (v > kGoClear || v != v) ? 1 : 2;  // NaN: the reference's !EPSLE(m, NaN) holds
}

// Row-side infeasibility: the reference's isConsInfeasible
// (src/propagation_methods.cuh:156-159, minact > rhs or maxact < lhs), taken
// only on a side with a finite constraint side and no infinite contribution,
// and with the relative tolerance of var_infeasible: an absolute EPS would
// flag feasible rows whose FP64 activities (terms up to 1e5, thousands of
// them) carry rounding errors of that size.
__device__ __forceinline__ bool row_infeasible(double minact, double maxact, int minf, int maxf, double lhs,
                                               double rhs) {
    if (minf == 0 && !is_posinf(rhs)) {
        double s = fmax(fabs(minact), fabs(rhs));
        if (s < 1.0) s = 1.0;
        if (dsub(minact, rhs) > dmul(kFeasTol, s)) return true;
    }
    if (maxf == 0 && !is_neginf(lhs)) {
        double s = fmax(fabs(maxact), fabs(lhs));
        if (s < 1.0) s = 1.0;
        if (dsub(lhs, maxact) > dmul(kFeasTol, s)) return true;
    }
    return false;
}

// ---- FP32 row screen -------------------------------------------------------
// Before any FP64 work a row is screened with FP32 interval arithmetic: an
// enclosure of the FP64 activities the exact pass would compute, the same
// infinity counts, and an upper bound U' >= U of the row filter's FP32 bound.
// A row the screen proves skippable is skipped by the exact rule too, so the
// screen changes no result; it only saves FP64 work on rows that cannot
// tighten anything (most of the non-zeros of a round on wide rows).
//
// Double -> float magnitude enclosure by integer work: truncation of the
// mantissa gives dn <= |x|, one float ulp more gives up >= |x|; magnitudes
// below 2^-126 enclose as [0, 2^-126], at or above 2^128 as [FLT_MAX, inf].
struct MagEnc {
    float dn, up;
};
__device__ __forceinline__ MagEnc mag_enc(long long bits) {
    const unsigned long long mag = (unsigned long long)bits & 0x7FFFFFFFFFFFFFFFULL;
    const unsigned hi = (unsigned)(mag >> 32);
    // low 32 bits of (mag >> 29) - (896 << 23): the float bit pattern when in range
    const unsigned fb = __funnelshift_r((unsigned)mag, hi, 29) - (896u << 23);
    MagEnc e;
    if (hi < (897u << 20)) {
        e.dn = 0.0f;
        e.up = __uint_as_float(0x00800000u);
    } else if (hi >= (1151u << 20)) {
        e.dn = __uint_as_float(0x7F7FFFFFu);
        e.up = __uint_as_float(0x7F800000u);
    } else {
        e.dn = __uint_as_float(fb);
        e.up = __uint_as_float(fb + 1u);
    }
    return e;
}

// The screen reads FP32 copies of the data (4 B per coefficient, 8 B per
// bound pair instead of 8 B and 16 B) that are made once: coefficients when
// the layout is built, bounds when a variable changes. Each copy is the
// round-to-nearest float, with these exceptions:
//  * a bound the reference counts as infinite (lb <= -1e20, ub >= 1e20) is
//    -inf / +inf, so the screen's infinity counts are the reference's;
//  * a finite bound above 2^100 in magnitude is NaN;
//  * a coefficient in (0, 1e-9] is NaN (the reference classifies it as
//    non-positive but sums it as positive), one above 2^40 in magnitude is
//    +-inf, and a non-zero one below 2^-60 in magnitude is NaN.
// NaN or inf terms make the screen's sums, magnitude sum or U NaN or inf,
// and every such row is left to the exact pass; the sign test a32 > 0 equals
// the reference's EPSGT(a, 0) for every coefficient, and a NaN copy keeps the
// coefficient's sign (so the sign bit tells a > 0, as in candidate_sides).
constexpr float kF32Inf = __builtin_huge_valf();
__host__ __device__ __forceinline__ float coef_screen(double a) {
    const double m = a < 0 ? -a : a;
    if (a > 0.0 && a <= kEps) return __builtin_nanf("");
    if (m > 0x1p40) return a > 0 ? kF32Inf : -kF32Inf;
    if (m != 0.0 && m < 0x1p-60) return a > 0 ? __builtin_nanf("") : -__builtin_nanf("");
    return (float)a;
}
constexpr long long kBits2p100 = 0x4630000000000000LL;  // 2^100
__device__ __forceinline__ float2 bnd_screen(double2 b) {
    const long long lb = dbits(b.x), ub = dbits(b.y);
    float2 r;
    r.x = neginf_bits(lb) ? -kF32Inf
          : (lb & 0x7FFFFFFFFFFFFFFFLL) > kBits2p100 ? __int_as_float(0x7FC00000) : __double2float_rn(b.x);
    r.y = posinf_bits(ub) ? kF32Inf
          : (ub & 0x7FFFFFFFFFFFFFFFLL) > kBits2p100 ? __int_as_float(0x7FC00000) : __double2float_rn(b.y);
    return r;
}

// max / min that return NaN when either operand is NaN (fmaxf drops it).
__device__ __forceinline__ float fmax_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float fmin_nan(float a, float b) {
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// Screen accumulator over the FP32 copies: mn / mx are round-to-nearest sums
// of the finite activity terms t = fl(a32 * b32), S >= the sum of their
// magnitudes (rounded upwards), U >= every |a| (ub - lb) up to a relative
// 2^-20 (see scr_u_bound), minf / maxf the reference's infinity counts.
//
// Error bound of the sums (Higham, Accuracy and Stability of Numerical
// Algorithms, 2nd ed., 3.1 and 4.2): each copy carries a relative error of
// at most u = 2^-24 and the product one more, so |t - a b| <= gamma_3 |t| /
// (1 - gamma_3); any summation order of n terms adds at most gamma_{n-1}
// sum |t|; the FP64 sums the exact pass computes (any order) are within
// gamma_n^(64) sum |a b| of the real sum. Together, for n <= 2^16,
// |minact_FP64 - mn| <= (n + 4) u (1 + 2^-6) S, and for n <= 2^20 with the
// factor 1.125; values below 2^-126 contribute absolute errors under 2^-80
// in total (|a32| <= 2^40). Rows longer than 2^20 are never skipped.
struct Scr {
    float mn, mx, S, U;
    int minf, maxf;
};
__device__ __forceinline__ void scr_init(Scr &c) {
    c.mn = 0.0f; c.mx = 0.0f; c.S = 0.0f; c.U = 0.0f;
    c.minf = 0; c.maxf = 0;
}
// One element: coefficient copy a, bound copies b = (lb, ub).
__device__ __forceinline__ void scr_add(Scr &c, float a, float2 b) {
    const bool pos = a > 0.0f;
    const float bmin = pos ? b.x : b.y, bmax = pos ? b.y : b.x;
    const bool imin = fabsf(bmin) == kF32Inf, imax = fabsf(bmax) == kF32Inf;
    c.minf += imin;
    c.maxf += imax;
    const float tmin = imin ? 0.0f : __fmul_rn(a, bmin);
    const float tmax = imax ? 0.0f : __fmul_rn(a, bmax);
    c.mn = __fadd_rn(c.mn, tmin);
    c.mx = __fadd_rn(c.mx, tmax);
    c.S = __fadd_ru(c.S, __fadd_ru(fabsf(tmin), fabsf(tmax)));
    // |a| (ub - lb) <= |a32| (fl(ub32 - lb32) + 2^-21 fl(|ub32| + |lb32|)) up
    // to a relative 2^-21: the copies' errors are at most 2^-24 of |ub|, |lb|
    const float d = __fsub_rn(b.y, b.x), w = __fadd_rn(fabsf(b.y), fabsf(b.x));
    c.U = fmax_nan(c.U, __fmul_rn(fabsf(a), __fmaf_rn(w, 0x1p-21f, d)));
}
__device__ __forceinline__ void scr_combine(Scr &a, const Scr &b) {
    a.mn = __fadd_rn(a.mn, b.mn);
    a.mx = __fadd_rn(a.mx, b.mx);
    a.S = __fadd_ru(a.S, b.S);
    a.U = fmax_nan(a.U, b.U);
    a.minf += b.minf;
    a.maxf += b.maxf;
}
// Largest float not above 1e20 (the infinity threshold).
constexpr float kInfF32Dn = 0x1.5af1d6p+66f;
// Upper bound of every FP64 |a| (ub - lb) of the row (each fl(|a| fl(ub - lb)),
// and so of the reference's sequential maxactdelta), the row filter's U: the
// accumulated U widened by 2^-20 relative plus 2^-80 absolute (bounds below
// 2^-126).
__device__ __forceinline__ float scr_u_bound(const Scr &c) { return __fmaf_ru(c.U, kUMargin, 0x1p-80f); }
// Enclosure [mn_lo, mn_hi] of min(rhs - minact, maxact - lhs) as the exact
// pass computes it in FP64 for a row of n elements: the activities lie within
// E of mn / mx, and FP64 rounding of the differences is monotone.
__device__ __forceinline__ void scr_slack(const Scr &c, int n, double lhs, double rhs, float &mn_lo,
                                          float &mn_hi) {
    const float k = n <= (1 << 20) ? __fmul_ru((float)(n + 4), n <= (1 << 16) ? 0x1.04p-24f : 0x1.2p-24f)
                                   : kF32Inf;
    const float E = __fmaf_ru(c.S, k, 0x1p-80f);
    const MagEnc R = mag_enc(dbits(rhs)), Lh = mag_enc(dbits(lhs));
    const bool rsg = dbits(rhs) < 0, lsg = dbits(lhs) < 0;
    const float rhs_dn = rsg ? -R.up : R.dn, rhs_up = rsg ? -R.dn : R.up;
    const float lhs_dn = lsg ? -Lh.up : Lh.dn, lhs_up = lsg ? -Lh.dn : Lh.up;
    const float s_lo = __fsub_rd(rhs_dn, __fadd_ru(c.mn, E));
    const float s_hi = __fsub_ru(rhs_up, __fsub_rd(c.mn, E));
    const float t_lo = __fsub_rd(__fsub_rd(c.mx, E), lhs_up);
    const float t_hi = __fsub_ru(__fadd_ru(c.mx, E), lhs_dn);
    mn_lo = fmin_nan(s_lo, t_lo);
    mn_hi = fminf(s_hi, t_hi);  // min(s, t) <= either upper end
}
// FP32 enclosure lo <= fl(|a| fl(ub - lb)) <= hi of one element from the
// screen copies (the copies' errors as in scr_add, widened by 2^-20 relative
// and 2^-80 absolute, which also covers the two FP64 roundings). A bound coded
// +-inf is at least 1e20 in magnitude, so the lower end uses +-kInfF32Dn in its
// place; NaN copies leave both ends NaN, and the comparisons then stay open.
__device__ __forceinline__ DeltaBox delta_box32(float a, float2 b) {
    const float aa = fabsf(a);
    const float d = __fsub_rn(b.y, b.x), w = __fadd_rn(fabsf(b.y), fabsf(b.x));
    DeltaBox r;
    r.hi = __fmaf_ru(__fmul_rn(aa, __fmaf_rn(w, 0x1p-21f, d)), kUMargin, 0x1p-80f);
    const float ubl = fmin_nan(b.y, kInfF32Dn), lbh = fmax_nan(b.x, -kInfF32Dn);
    const float dl = __fsub_rn(ubl, lbh), wl = __fadd_rn(fabsf(ubl), fabsf(lbh));
    r.lo = __fmaf_rd(__fmul_rn(fmin_nan(aa, 0x1p40f), __fmaf_rn(wl, -0x1p-21f, dl)), 0.99999904632568359375f,
                     -0x1p-80f);
    return r;
}

// True when the reference's row test certainly skips the row, whatever order
// the exact pass sums it in: its sequential maxactdelta is at most the largest
// FP64 |a| (ub - lb), which the widened U bounds, and U <= min slack. Such a
// row is not infeasible either (both slacks are >= 0).
__device__ __forceinline__ bool scr_skips(const Scr &c, int n, double lhs, double rhs) {
    if (c.minf > 1 && c.maxf > 1) return true;
    float mn_lo, mn_hi;
    scr_slack(c, n, lhs, rhs, mn_lo, mn_hi);
    return mn_hi < kInfF32Dn && __fmul_ru(scr_u_bound(c), kUMargin) <= mn_lo;
}

// The certified margin of a row the screen skips (scr_skips): how far the
// row's FP64 slacks may still fall, whatever order they are summed in, before
// that skip's certificate fails -- every |a| (ub - lb) only shrinks as bounds
// tighten, so the certificate u <= slack needs the slacks alone. It is mn_lo -
// u (u = fl_ru(U kUMargin)), less 2^-30 S for the FP64 summation errors of
// the certifying and of a later evaluation (n <= 2^20 terms, 2^-33 S each,
// with S grown by the drift at most), 2^-50 |mn_lo| for the rounding of the
// slack itself and 2^-80, rounded down. A row skipped on its infinite
// contributions keeps its skip until a bound becomes finite (an infinite
// drift): margin DBL_MAX. -1 when the screen does not skip the row.
__device__ __forceinline__ double scr_margin(const Scr &c, int n, double lhs, double rhs) {
    if (c.minf > 1 && c.maxf > 1) return 1.7976931348623157e308;
    float lo, hi;
    scr_slack(c, n, lhs, rhs, lo, hi);
    const float u = __fmul_ru(scr_u_bound(c), kUMargin);
    if (!(hi < kInfF32Dn && u <= lo)) return -1.0;
    double m = __dsub_rd((double)lo, (double)u);
    m = __dsub_rd(m, __dmul_ru((double)c.S, 0x1p-30));
    m = __dsub_rd(m, __dmul_ru(fabs((double)lo), 0x1p-50));
    return __dsub_rd(m, 0x1p-80);
}

// The project's infeasibility rule (the reference detects none).
__device__ __forceinline__ bool var_infeasible(double lb, double ub) {
    double s = fmax(fabs(lb), fabs(ub));
    if (s < 1.0) s = 1.0;
    return dsub(lb, ub) > dmul(kFeasTol, s);
}

}  // namespace gdp

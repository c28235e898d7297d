// gdp_round.cuh -- the device side of one Jacobi propagation round, shared
// by the single-problem kernels (gdp_round.cu) and the batched engine
// (gdp_batch.cu).
//
// A round reads the round-start bounds (cur), writes every tightening into nxt
// with an FP64 min/max atomic and flags the variable in a bitmap; the finalize
// phase copies flagged variables nxt -> cur, applies the infeasibility rule
// and marks the rows of changed variables for the next round. The result does
// not depend on scheduling: each row's sums run in a fixed order from the
// snapshot and min/max commute.
//
// GB300's FP64 pipe (about 1.75 lane-ops per clock per SM) is the scarce
// resource, so the kernels spend it only on the reference's arithmetic: 2 DMUL
// + 2 DADD per non-zero for the activities, and only on rows that an FP32
// interval screen could not prove skippable. Classification against the
// +-1e20 infinity thresholds is integer work on the bit patterns, the
// reference's row test (canConsBeTightened) is pre-filtered with an FP32 upper
// bound of max |a|(ub - lb) and decided exactly only for rows that survive,
// and the candidate divisions of a warp are gathered into a queue and run 32
// at a time instead of diverging.
//
// Reference: the round body of GPUAtomicDomainPropagation
// (src/kernels/atomic_kernel.cuh:9-450) and of the megakernel
// (src/kernels/atomic_megakernel.cuh:14-490), re-planned for a snapshot
// schedule; math from src/propagation_methods.cuh:78-276.
#pragma once

#include <climits>
#include <cuda_runtime.h>

#include "gdp_device.cuh"
#include "gdp_internal.h"

namespace gdp {
namespace {


constexpr unsigned kFull = 0xffffffffu;
constexpr int kQueueCap = 128;  // >= 31 pending + 64 pushed per step

// Phase timers, compiled only into a library built with -DGDP_PHASE_TIMERS
// (build.py --phase-timers): the megakernel stamps %globaltimer at the start of
// each round and after each of its grid barriers, every warp adds the time it
// spends in each phase, and the exact pass of SELL rows adds its two passes'
// warp time by lane-group size. In the plain build timer_now() is 0 and the
// recording calls are empty.
constexpr int kTimerRounds = 1024;  // rounds recorded (later rounds are not)
constexpr int kTimerSlots = 8;      // per round: 5 stamps + 3 work counters; 5 phase busy sums
constexpr int kTimerPass = 16;      // 2 passes x lane-group sizes 1..32, then one-lane row work
#ifdef GDP_PHASE_TIMERS
__device__ unsigned long long g_timer_wall[kTimerRounds * kTimerSlots];
__device__ unsigned long long g_timer_busy[kTimerRounds * kTimerSlots];
__device__ unsigned long long g_timer_pass[kTimerPass];
__device__ __forceinline__ unsigned long long timer_now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// warp time of the exact pass's pass 1 [t0, t1) and pass 2 [t1, now)
__device__ __forceinline__ void timer_pass(int lane, int lg, unsigned long long t0, unsigned long long t1) {
    if (lane == 0) {
        const unsigned long long t2 = timer_now();
        atomicAdd(&g_timer_pass[2 * lg], t1 - t0);
        atomicAdd(&g_timer_pass[2 * lg + 1], t2 - t1);
    }
}
// one-lane rows of an exact-pass warp: their elements (slot 12) against 32 x
// the longest (slot 13), the lane utilisation of the row loops
__device__ __forceinline__ void timer_lanes(int lane, int lg, int cnt) {
    if (lg != 0) return;
    int sum = cnt, mx = cnt;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, off);
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if (lane == 0) {
        atomicAdd(&g_timer_pass[12], (unsigned long long)sum);
        atomicAdd(&g_timer_pass[13], 32ull * (unsigned long long)mx);
    }
}
#else
__device__ __forceinline__ unsigned long long timer_now() { return 0ull; }
__device__ __forceinline__ void timer_pass(int, int, unsigned long long, unsigned long long) {}
__device__ __forceinline__ void timer_lanes(int, int, int) {}
#endif

__device__ __forceinline__ void mark_changed(const DevProblem &P, int j) {
    atomicOr(P.chg + (j >> 5), 1u << (j & 31));
}

// Bounds are written by the finalize phase of the same megakernel launch, so
// they are read with coherent loads (never the read-only path).
__device__ __forceinline__ double2 load_bnd(const DevProblem &P, int j) { return P.bnd[j]; }
// The layout of bnd32 is fixed per kernel: kRec = 1, the stamped 16-byte
// records (BndScr) of single-problem contexts -- the round loops of the
// megakernel, the phase kernels and learned marking; kRec = 0, the 8-byte
// copies of batch members.
// Variable j's screen copy of its bounds.
template <int kRec>
__device__ __forceinline__ float2 load_bnd32(const DevProblem &P, int j) {
    return P.bnd32[kRec ? 2 * (long long)j : j];
}
// The screen copy of variable j's bounds, with chg set when the variable was
// committed at the end of the round before `round` (one 16-byte load of the
// stamped record; copies without stamps leave chg alone).
template <int kRec>
__device__ __forceinline__ float2 load_bnd32_chg(const DevProblem &P, int j, int round, int &chg) {
    if (!kRec) return P.bnd32[j];
    const float4 v = reinterpret_cast<const float4 *>(P.bnd32)[j];
    chg |= __float_as_int(v.z) == round - 1 ? 1 : 0;
    return make_float2(v.x, v.y);
}
// Stores variable j's screen copy of bounds b committed at the end of `round`.
template <int kRec>
__device__ __forceinline__ void store_bnd32(const DevProblem &P, int j, double2 b, int round) {
    const float2 f = bnd_screen(b);
    if (kRec) reinterpret_cast<float4 *>(P.bnd32)[j] = make_float4(f.x, f.y, __int_as_float(round), 0.0f);
    else P.bnd32[j] = f;
}
// Whether a row the screen cannot skip takes the exact pass in `round`: a row
// none of whose variables changed at the end of the previous round (chg == 0)
// was last processed with the same bounds, so its activities and candidates
// are those of that processing -- applied then, or not EPS-better than bounds
// that have not moved since -- and it can neither tighten a bound nor turn
// infeasible. Round 1 processes every row. Valid where every row with a
// changed variable is processed in the next round (full sweeps and exact
// marking): not under learned deferral, and only with stamped records.
template <int kRec>
__device__ __forceinline__ bool row_due(const DevProblem &P, int round, int chg) {
    return chg != 0 || round <= 1 || !kRec || P.learned != 0;
}

// Row constants of tightenVariable (src/propagation_methods.cuh:223-276), with
// float thresholds that decide most per-element EPS tests without FP64:
// d <= x if d_hi <= f32_dn(x); fl(d - x) > 1e-9 if d_lo > f32_up(fl(x + 4e-9))
// (then d - x > 3e-9 for |x| < 2^24, and d > x with ulp(x) > 3.7e-9 above).
struct RowC {
    double slack, surplus;  // rhs - minact, lhs - maxact
    double neg_surplus;     // maxact - lhs
    int minf, maxf;
    int ok;                 // bit 0: rhs side usable, bit 1: lhs side usable
    float slack_dn, slack_hi, nsur_dn, nsur_hi;
};

__device__ __forceinline__ RowC make_rowc(double minact, double maxact, int minf, int maxf, double lhs,
                                          double rhs) {
    RowC c;
    c.slack = dsub(rhs, minact);
    c.surplus = dsub(lhs, maxact);
    c.neg_surplus = dsub(maxact, lhs);
    c.minf = minf;
    c.maxf = maxf;
    const bool rhs_ok = !posinf_bits(dbits(rhs)) && !neginf_bits(dbits(minact));
    const bool lhs_ok = !neginf_bits(dbits(lhs)) && !posinf_bits(dbits(maxact));
    c.ok = (rhs_ok ? 1 : 0) | (lhs_ok ? 2 : 0);
    c.slack_dn = f32_dn(dbits(c.slack));
    c.slack_hi = f32_up(dbits(dadd(c.slack, 4e-9)));
    c.nsur_dn = f32_dn(dbits(c.neg_surplus));
    c.nsur_hi = f32_up(dbits(dadd(c.neg_surplus, 4e-9)));
    return c;
}

// 0: EPSGT(d, x) is false, 1: true, 2: undecided from the enclosure.
__device__ __forceinline__ int side_test(const DeltaBox &b, float x_dn, float x_hi) {
    if (b.hi <= x_dn) return 0;
    if (b.lo > x_hi) return 1;
    return 2;
}

// Which candidate sides of element (a, lb, ub) need a division. Bit 0: upper
// bound (tightenVarUpperBound), bit 1: lower bound (tightenVarLowerBound).
// The FP64 product |a|(ub-lb) -- equal bit for bit to the reference's
// coeff*(ub-lb) / coeff*(lb-ub) -- is formed only when the enclosure leaves a
// test undecided.
__device__ __forceinline__ int candidate_sides(const RowC &c, double a, double lb, double ub) {
    const long long ab = dbits(a), lbb = dbits(lb), ubb = dbits(ub);
    const DeltaBox box = delta_box(ab, lbb, ubb);
    int rs = (c.ok & 1) ? side_test(box, c.slack_dn, c.slack_hi) : 0;
    int ls = (c.ok & 2) ? side_test(box, c.nsur_dn, c.nsur_hi) : 0;
    if (rs == 2 || ls == 2) {
        const double d = dmul(fabs(a), dsub(ub, lb));
        if (rs == 2) rs = eps_gt_fast(d, c.slack) ? 1 : 0;
        if (ls == 2) ls = eps_gt_fast(d, c.neg_surplus) ? 1 : 0;
    }
    const bool pos = gt0_bits(ab);
    const bool u_side = pos ? rs : ls;
    const bool l_side = pos ? ls : rs;
    const int nu = pos ? c.minf : c.maxf;
    const int nl = pos ? c.maxf : c.minf;
    const bool u_ok = u_side && (nu == 0 || (nu == 1 && neginf_bits(lbb)));
    const bool l_ok = l_side && (nl == 0 || (nl == 1 && posinf_bits(ubb)));
    return (u_ok ? 1 : 0) | (l_ok ? 2 : 0);
}

// candidate_sides from the screen copies of the coefficient and the bounds.
// Returns 4 when the FP32 box leaves a side test open; the caller then decides
// with the FP64 values (candidate_sides). Signs and infinity tests are exact on
// the copies: the sign bit of a32 is a's, and -inf / +inf copies are exactly
// the bounds the reference counts as infinite.
__device__ __forceinline__ int candidate_sides32(const RowC &c, float a, float2 b) {
    const DeltaBox box = delta_box32(a, b);
    const int rs = (c.ok & 1) ? side_test(box, c.slack_dn, c.slack_hi) : 0;
    const int ls = (c.ok & 2) ? side_test(box, c.nsur_dn, c.nsur_hi) : 0;
    if (rs == 2 || ls == 2) return 4;
    const bool pos = __float_as_int(a) > 0;
    const bool u_side = pos ? rs : ls;
    const bool l_side = pos ? ls : rs;
    const int nu = pos ? c.minf : c.maxf;
    const int nl = pos ? c.maxf : c.minf;
    const bool u_ok = u_side && (nu == 0 || (nu == 1 && b.x == -kF32Inf));
    const bool l_ok = l_side && (nl == 0 || (nl == 1 && b.y == kF32Inf));
    return (u_ok ? 1 : 0) | (l_ok ? 2 : 0);
}

// One candidate (side 0: upper, 1: lower) of variable j; applies it with an
// FP64 atomic if EPS-better than the snapshot. Returns true if it tightened.
// b: the variable's round-start bounds (read-only during the round).
__device__ __forceinline__ bool apply_side(const DevProblem &P, const RowC &c, int j, double a, double2 b,
                                           int side) {
    const bool pos = gt0_bits(dbits(a));
    const bool cont = __ldg(P.is_cont + j) != 0;
    if (side == 0) {
        const int ninf = pos ? c.minf : c.maxf;
        double nb = ddiv(pos ? c.slack : c.surplus, a);
        if (ninf == 0) nb = dadd(nb, b.x);
        if (!cont) nb = eps_floor(nb);
        if (eps_lt(nb, b.y)) {
            atomic_min_f64(&P.bnd_nxt[j].y, nb);
            mark_changed(P, j);
            return true;
        }
    } else {
        const int ninf = pos ? c.maxf : c.minf;
        double nb = ddiv(pos ? c.surplus : c.slack, a);
        if (ninf == 0) nb = dadd(nb, b.y);
        if (!cont) nb = eps_ceil(nb);
        if (eps_gt(nb, b.x)) {
            atomic_max_f64(&P.bnd_nxt[j].x, nb);
            mark_changed(P, j);
            return true;
        }
    }
    return false;
}

// ---- warp division queue --------------------------------------------------
// A queued candidate side carries its variable and its position (element
// index, owner lane, side), so draining it reloads the coefficient and the
// bounds with two independent loads (no column -> bound chain). push()
// appends each lane's sides (ballot + prefix), drain() runs batches of 32.
struct QEntry {  // 8 bytes
    int j;
    unsigned code;  // bit 0: side (0 upper, 1 lower); bits 1..5: owner lane; bits 6..: element step
};

struct WarpQueue {
    QEntry *q;
    int cnt;     // warp-uniform
    int pushed;  // warp-uniform: candidate sides queued (each one division)
};

template <class Run>
__device__ __forceinline__ void queue_drain(WarpQueue &Q, int lane, bool all, Run &&run) {
    while (Q.cnt >= 32 || (all && Q.cnt > 0)) {
        const int take = Q.cnt < 32 ? Q.cnt : 32;
        if (lane < take) run(Q.q[lane]);
        __syncwarp();
        const int rest = Q.cnt - take;
        for (int i = lane; i < rest; i += 32) Q.q[i] = Q.q[take + i];
        __syncwarp();
        Q.cnt = rest;
    }
}

__device__ __forceinline__ void queue_push(WarpQueue &Q, int lane, int sides, int j, unsigned code_base) {
    const unsigned bu = __ballot_sync(kFull, sides & 1);
    const unsigned bl = __ballot_sync(kFull, sides & 2);
    const unsigned lt = (1u << lane) - 1u;
    if (sides & 1) Q.q[Q.cnt + __popc(bu & lt)] = QEntry{j, code_base};
    if (sides & 2) Q.q[Q.cnt + __popc(bu) + __popc(bl & lt)] = QEntry{j, code_base | 1u};
    __syncwarp();
    Q.cnt += __popc(bu) + __popc(bl);
    Q.pushed += __popc(bu) + __popc(bl);
}

// Warp-aggregated round bookkeeping: change flag and tightening count.
__device__ __forceinline__ void report_tight(int tight, int lane, int *change, unsigned *tight_ctr) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) tight += __shfl_down_sync(kFull, tight, off);
    if (lane == 0 && tight) {
        *change = 1;
        atomicAdd(tight_ctr, (unsigned)tight);
    }
}

// ---- SELL-g rows: one warp per slice, g lanes per row ----------------------
struct WarpSmem {
    RowC rc[32];
    QEntry q[kQueueCap];
    long long base[32];  // deferred exact pass: first element of each lane
    // work statistics of this warp, written by lane 0 and flushed to the
    // round flags once per phase (not once per item: same-address atomics
    // from every warp for every item would serialise in L2)
    unsigned long long st_rows, st_nnz, st_exact, st_div, st_xrows, st_go, st_seq, st_drift, st_drift_nnz;
};

__device__ __forceinline__ void stats_zero(WarpSmem &ws, int lane) {
    if (lane == 0) {
        ws.st_rows = 0; ws.st_nnz = 0; ws.st_exact = 0; ws.st_div = 0;
        ws.st_xrows = 0; ws.st_go = 0; ws.st_seq = 0; ws.st_drift = 0; ws.st_drift_nnz = 0;
    }
}
__device__ __forceinline__ void stats_flush(const DevProblem &P, WarpSmem &ws, int lane) {
    if (lane == 0) {
        if (ws.st_rows) atomicAdd(&P.flags[0].rows_proc, ws.st_rows);
        if (ws.st_nnz) atomicAdd(&P.flags[0].nnz_proc, ws.st_nnz);
        if (ws.st_exact) atomicAdd(&P.flags[0].nnz_exact, ws.st_exact);
        if (ws.st_div) atomicAdd(&P.flags[0].divisions, ws.st_div);
        if (ws.st_xrows) atomicAdd(&P.flags[0].rows_exact, ws.st_xrows);
        if (ws.st_go) atomicAdd(&P.flags[0].rows_go, ws.st_go);
        if (ws.st_seq) atomicAdd(&P.flags[0].rows_seqmax, ws.st_seq);
        if (ws.st_drift) atomicAdd(&P.flags[0].rows_drift, ws.st_drift);
        if (ws.st_drift_nnz) atomicAdd(&P.flags[0].nnz_drift, ws.st_drift_nnz);
        ws.st_rows = 0; ws.st_nnz = 0; ws.st_exact = 0; ws.st_div = 0;
        ws.st_xrows = 0; ws.st_go = 0; ws.st_seq = 0; ws.st_drift = 0; ws.st_drift_nnz = 0;
    }
}

// A row whose activities exclude [lhs, rhs] (row_infeasible): only its index is
// recorded here; the finalize step of the round turns it into the verdict, so
// that every driver completes the round as the oracle does.
__device__ __forceinline__ void record_row_infeasible(const DevProblem &P, int pos) {
    atomicMin(&P.flags[0].infeasible_row, __ldg(P.pos_row + pos));
}

// ---- the reference's sequential EPS-max, for rows row_go_from_max leaves open
// First maximum (order key, index) of d_k = fl(|a_k| fl(ub - lb)) over the
// elements [0, e) of a row stored contiguously at (col, val), with the
// leading 0.0 at index -1; NaN terms never count. All 32 lanes call it and
// every lane returns the result (a butterfly of an associative selection).
__device__ __forceinline__ void row_first_max(const DevProblem &P, const int *col, const double *val, int e,
                                              int lane, long long &km, int &p) {
    Acc s;
    acc_init(s);
    for (int k = lane; k < e; k += 32) {
        const double2 b = load_bnd(P, __ldg(col + k));
        acc_add_delta(s, dmul(fabs(__ldg(val + k)), dsub(b.y, b.x)), k);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const long long ok = __shfl_xor_sync(kFull, s.km, off);
        const int op = __shfl_xor_sync(kFull, s.p, off);
        acc_take_max(s, ok, op);
    }
    km = s.km;
    p = s.p;
}

// The reference's sequential EPS-max of the row's elements [0, len)
// (computeActivities, src/propagation_methods.cuh:188-190), given the first
// maximum (km, p) of [0, len). Over a prefix [0, E) with first maximum (M, q),
// m(E) = fl(M - m(q)) > EPS ? M : m(q) (row_go_from_max), and m(E) = M outright
// when the first maximum M' of [0, q) has fl(M - M') > EPS; m = 0 when the
// maximum is the leading 0.0. The prefix maxima are warp passes; their values
// wait in a stack of one level per lane. A chain deeper than 32 levels (values
// each within EPS of the next) ends with a serial scan. All 32 lanes call it.
__device__ __noinline__ double seq_eps_max(const DevProblem &P, const int *col, const double *val, int len,
                                           long long km, int p, int lane) {
    double stack = 0.0;
    int depth = 0, E = len;
    double x = 0.0;
    for (;;) {
        if (p < 0) {
            x = 0.0;
            break;
        }
        const double M = __longlong_as_double(km);
        if (depth == 32) {
            double m = 0.0;
            if (lane == 0)
                for (int k = 0; k < E; k++) {
                    const double2 b = load_bnd(P, __ldg(col + k));
                    const double d = dmul(fabs(__ldg(val + k)), dsub(b.y, b.x));
                    if (eps_gt(d, m)) m = d;
                }
            x = __shfl_sync(kFull, m, 0);
            break;
        }
        if (lane == depth) stack = M;
        depth++;
        long long km2;
        int p2;
        row_first_max(P, col, val, p, lane, km2, p2);
        if (p2 >= 0 && eps_gt(M, __longlong_as_double(km2))) {
            depth--;  // m(E) = M
            x = M;
            break;
        }
        E = p;
        km = km2;
        p = p2;
    }
    for (int i = depth - 1; i >= 0; i--) {
        const double Mi = __shfl_sync(kFull, stack, i);
        if (eps_gt(Mi, x)) x = Mi;
    }
    return x;
}

// Warp-level dynamic work counter that keeps the next claim in flight while
// the current item is processed: the contended atomic's round trip overlaps
// with useful work instead of stalling the warp between items.
struct WarpCursor {
    unsigned *ctr;
    unsigned step;
    unsigned pre;  // lane 0: the claim in flight
    __device__ __forceinline__ void start(unsigned *c, unsigned stp, int lane) {
        ctr = c;
        step = stp;
        pre = 0;
        if (lane == 0) pre = atomicAdd(c, stp);
    }
    __device__ __forceinline__ int next(int lane) {
        const int i = (int)__shfl_sync(kFull, pre, 0);
        if (lane == 0) pre = atomicAdd(ctr, step);
        return i;
    }
};

// Learned marking: scores and per-row outcomes of one slice (the features
// of the slice's rows live in the warp's division-queue storage, which is
// free until the exact pass).
struct LearnSmem {
    float z[32];
    int tight[32];
    int go[32];
    unsigned long long marked;  // marked SELL rows met by this warp in the current phase
};

// Combines the partial accumulators of a group of g lanes (g a power of two,
// warp-uniform) into its first lane: shuffle tree with offsets g/2, ..., 1.
__device__ __forceinline__ void acc_group_reduce(Acc &s, int g) {
    for (int off = g >> 1; off > 0; off >>= 1) {
        Acc o;
        o.minact = __shfl_down_sync(kFull, s.minact, off);
        o.maxact = __shfl_down_sync(kFull, s.maxact, off);
        o.minf = __shfl_down_sync(kFull, s.minf, off);
        o.maxf = __shfl_down_sync(kFull, s.maxf, off);
        o.km = __shfl_down_sync(kFull, s.km, off);
        o.p = __shfl_down_sync(kFull, s.p, off);
        acc_combine(s, o);
    }
}

__device__ __forceinline__ void scr_group_reduce(Scr &c, int g) {
    for (int off = g >> 1; off > 0; off >>= 1) {
        Scr o;
        o.mn = __shfl_down_sync(kFull, c.mn, off);
        o.mx = __shfl_down_sync(kFull, c.mx, off);
        o.S = __shfl_down_sync(kFull, c.S, off);
        o.U = __shfl_down_sync(kFull, c.U, off);
        o.minf = __shfl_down_sync(kFull, c.minf, off);
        o.maxf = __shfl_down_sync(kFull, c.maxf, off);
        scr_combine(c, o);
    }
}

// Adds the warp's row and non-zero counts to the round statistics.
__device__ __forceinline__ void count_work(WarpSmem &ws, int lane, int rows, int nnz, int nnz_exact) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rows += __shfl_down_sync(kFull, rows, off);
        nnz += __shfl_down_sync(kFull, nnz, off);
        nnz_exact += __shfl_down_sync(kFull, nnz_exact, off);
    }
    if (lane == 0) {
        ws.st_rows += (unsigned long long)rows;
        ws.st_nnz += (unsigned long long)nnz;
        ws.st_exact += (unsigned long long)nnz_exact;
    }
}

// Where the exact pass finds a row's elements: step i of lane l at
// col[ws.base[l] + stride i] -- stride 32 in the SELL slices (a warp that
// screened the slice), stride g in the row-contiguous copy (the deferred
// pass, whose rows come from different slices: a lane's successive elements
// then share sectors instead of sitting 128 B / 256 B apart).
struct ElemView {
    const int *col;
    const double *val;
    const float *a32;  // screen copies of val (the candidate tests read these)
    int stride;
};
__device__ __forceinline__ ElemView sell_view(const DevProblem &P) {
    return ElemView{P.sell_col, P.sell_val, P.sell_a32, 32};
}

// Exact pass of up to 32/g SELL-g rows held by one warp, g lanes per row:
// lane l serves row l >> lg (active if `exact`), its elements at
// ws.base[l] + stride i for i < cnt (element sub + g i of the row, sub = l & (g-1)).
// The leader lane of each row (sub == 0) holds its position, lhs and rhs.
//   pass 1: exact FP64 activities. g == 1 rows are summed left to right,
//           with the reference's sequential EPS-max of |a|(ub - lb) in the
//           same loop; g > 1 rows are combined by a shuffle tree together
//           with the first FP64 maximum of |a|(ub - lb), from which
//           row_go_from_max takes the reference's decision (seq_eps_max over
//           the row-contiguous copy where it cannot). Every row takes the
//           reference's row test, and every row is checked for row-side
//           infeasibility.
//   pass 2: candidates through the warp division queue.
template <int kRec>
__device__ __forceinline__ void sell_rows_exact(const DevProblem &P, const ElemView ev, int lg, int lane,
                                                bool exact, int len,
                                                int cnt, double lhs, double rhs, int pos, float slack_lo,
                                                int *change,
                                                unsigned *tight_ctr, WarpSmem &ws, int *row_tight = nullptr,
                                                int *row_go = nullptr) {
    const unsigned long long t_pass0 = timer_now();
    const int g = 1 << lg;
    const int rl = lane >> lg, sub = lane & (g - 1);
    const bool leader = exact && sub == 0;
    const long long base = ws.base[lane];
    const int *col = ev.col + base;
    const double *val = ev.val + base;
    const int st = ev.stride;
    const int cnt1 = exact ? cnt : 0;
    timer_lanes(lane, lg, cnt1);
    Acc s;
    acc_init(s);
    double mn = 0.0;
    int dec = 0;
    unsigned cmask = lg == 0 ? 0u : (cnt1 >= 32 ? ~0u : (1u << cnt1) - 1u);
    if (lg == 0) {
        // one lane per row, elements in order: the reference's left-to-right
        // sums and its sequential EPS-max of |a|(ub - lb) in the same loop, so
        // the row test is the reference's own (canConsBeTightened)
        // cmask: the elements whose |a|(ub - lb) exceeds the screen's lower
        // bound of both slacks -- the only ones that can yield a candidate
        // (an integer compare of the keys; inf / NaN always pass)
        double m = 0.0;
        const long long kcut = order_key(dbits(slack_lo == slack_lo ? (double)slack_lo : -1e308));
        auto elem = [&](int i, double a, double2 b) {
            acc_add_terms(s, a, b.x, b.y);
            const double d = dmul(fabs(a), dsub(b.y, b.x));
            if (eps_gt_fast(d, m)) m = d;
            const long long db = dbits(d);
            if (order_key(db) > kcut || (db & 0x7FF0000000000000LL) == 0x7FF0000000000000LL)
                cmask |= 1u << (i & 31);
        };
        if (st == 1) {
            // the row-contiguous copy: rows start on 4-element boundaries and
            // are zero-padded to them, so 4 columns and 4 coefficients come in
            // three 16-byte loads and the 4 bound gathers go out together
            for (int i = 0; i < cnt1; i += 4) {
                const int4 c4 = __ldg(reinterpret_cast<const int4 *>(col + i));
                const double2 v01 = __ldg(reinterpret_cast<const double2 *>(val + i));
                const double2 v23 = __ldg(reinterpret_cast<const double2 *>(val + i + 2));
                const bool k1 = i + 1 < cnt1, k2 = i + 2 < cnt1, k3 = i + 3 < cnt1;
                const double2 b0 = load_bnd(P, c4.x);
                double2 b1 = make_double2(0.0, 0.0), b2 = b1, b3 = b1;
                if (k1) b1 = load_bnd(P, c4.y);
                if (k2) b2 = load_bnd(P, c4.z);
                if (k3) b3 = load_bnd(P, c4.w);
                elem(i, v01.x, b0);
                if (k1) elem(i + 1, v01.y, b1);
                if (k2) elem(i + 2, v23.x, b2);
                if (k3) elem(i + 3, v23.y, b3);
            }
        } else {
#pragma unroll 4
            for (int i = 0; i < cnt1; i++) {
                const int j = __ldg(col + st * i);
                elem(i, __ldg(val + st * i), load_bnd(P, j));
            }
        }
        if (leader) {
            mn = row_min_slack(s.minact, s.maxact, lhs, rhs);
            dec = reference_row_go(s.minf, s.maxf, m, mn) ? 1 : 0;
        }
    } else {
#pragma unroll 4
        for (int i = 0; i < cnt1; i++) {
            const int j = __ldg(col + st * i);
            const double a = __ldg(val + st * i);
            const double2 b = load_bnd(P, j);
            acc_add_terms(s, a, b.x, b.y);
            acc_add_delta(s, dmul(fabs(a), dsub(b.y, b.x)), sub + (i << lg));
        }
        acc_group_reduce(s, g);
        if (leader) {
            mn = row_min_slack(s.minact, s.maxact, lhs, rhs);
            dec = row_go_from_max(s.minf, s.maxf, acc_max(s), mn);
        }
        // rows whose test only the sequential EPS-max decides (the largest
        // |a| (ub - lb) exceeds the slack by EPS to 2.00001e-9): the warp
        // computes it row by row over the row-contiguous copy
        unsigned amb = __ballot_sync(kFull, leader && dec == 2);
        if (lane == 0) ws.st_seq += __popc(amb);
        while (amb) {
            const int src = __ffs(amb) - 1;
            amb &= amb - 1;
            const int apos = __shfl_sync(kFull, pos, src);
            const int alen = __shfl_sync(kFull, len, src);
            const long long akm = __shfl_sync(kFull, s.km, src);
            const int ap = __shfl_sync(kFull, s.p, src);
            const double amn = __shfl_sync(kFull, mn, src);
            const long long xb = __ldg(P.xptr + apos);
            const double m = seq_eps_max(P, P.xcol + xb, P.xval + xb, alen, akm, ap, lane);
            if (lane == src) dec = eps_le(m, amn) ? 0 : 1;
        }
    }
    if (leader && row_infeasible(s.minact, s.maxact, s.minf, s.maxf, lhs, rhs)) record_row_infeasible(P, pos);
    {
        const unsigned bx = __ballot_sync(kFull, leader);
        if (lane == 0) ws.st_xrows += __popc(bx);
    }
    const unsigned long long t_pass1 = timer_now();
    int tight = 0;
    const bool go = __shfl_sync(kFull, dec, rl << lg) == 1 && exact;
    if (row_go && leader) row_go[rl] = go ? 1 : 0;
    {
        const unsigned bg = __ballot_sync(kFull, go && sub == 0);
        if (lane == 0) ws.st_go += __popc(bg);
    }
    if (__any_sync(kFull, go)) {
        if (leader && dec == 1) ws.rc[rl] = make_rowc(s.minact, s.maxact, s.minf, s.maxf, lhs, rhs);
        __syncwarp();
        WarpQueue Q{ws.q, 0, 0};
        auto run = [&](const QEntry &q) {
            const int owner = (q.code >> 1) & 31;
            const int slot = owner >> lg;
            const double a = __ldg(ev.val + ws.base[owner] + (long long)st * (int)(q.code >> 6));
            if (apply_side(P, ws.rc[slot], q.j, a, load_bnd(P, q.j), (int)(q.code & 1u))) {
                tight++;
                if (row_tight) atomicAdd(row_tight + slot, 1);
            }
        };
        int maxcnt = go ? cnt : 0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) maxcnt = max(maxcnt, __shfl_xor_sync(kFull, maxcnt, off));
        // software pipeline over the screen copies: the element after next's
        // column and coefficient and the next element's bounds are in flight
        // while an element is tested; the FP64 values are read only for tests
        // the FP32 box leaves open. A lane visits the elements of cmask (all
        // of them for rows summed by several lanes).
        const float *a32 = ev.a32 + base;
        if (__all_sync(kFull, cnt1 <= 32)) {
            unsigned rem = go ? cmask : 0u;
            int nvis = __popc(rem);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) nvis = max(nvis, __shfl_xor_sync(kFull, nvis, off));
            int i1 = -1, i2 = -1, j1 = 0, j2 = 0;
            float a1 = 0.0f, a2 = 0.0f;
            float2 b1 = make_float2(0.0f, 0.0f);
            if (rem) { i1 = __ffs(rem) - 1; rem &= rem - 1; j1 = __ldg(col + st * i1); a1 = __ldg(a32 + st * i1); }
            if (rem) { i2 = __ffs(rem) - 1; rem &= rem - 1; j2 = __ldg(col + st * i2); a2 = __ldg(a32 + st * i2); }
            if (i1 >= 0) b1 = load_bnd32<kRec>(P, j1);
            for (int t = 0; t < nvis; t++) {
                const int i = i1, j = j1;
                const float a = a1;
                const float2 b = b1;
                i1 = i2; j1 = j2; a1 = a2;
                i2 = -1;
                if (rem) { i2 = __ffs(rem) - 1; rem &= rem - 1; j2 = __ldg(col + st * i2); a2 = __ldg(a32 + st * i2); }
                if (i1 >= 0) b1 = load_bnd32<kRec>(P, j1);
                int sides = i >= 0 ? candidate_sides32(ws.rc[rl], a, b) : 0;
                if (sides & 4) {
                    const double2 bd = load_bnd(P, j);
                    sides = candidate_sides(ws.rc[rl], __ldg(val + st * i), bd.x, bd.y);
                }
                queue_push(Q, lane, sides, j, ((unsigned)max(i, 0) << 6) | ((unsigned)lane << 1));
                queue_drain(Q, lane, false, run);
            }
        } else {  // a lane holds more than 32 elements (thread_row_max or split_tile raised): every element
            const int ce = go ? cnt : 0;
            int j1 = 0, j2 = 0;
            float a1 = 0.0f, a2 = 0.0f;
            float2 b1 = make_float2(0.0f, 0.0f);
            if (ce > 0) { j1 = __ldg(col); a1 = __ldg(a32); }
            if (ce > 1) { j2 = __ldg(col + st); a2 = __ldg(a32 + st); }
            if (ce > 0) b1 = load_bnd32<kRec>(P, j1);
            for (int i = 0; i < maxcnt; i++) {
                const int j = j1;
                const float a = a1;
                const float2 b = b1;
                j1 = j2;
                a1 = a2;
                if (i + 2 < ce) { j2 = __ldg(col + st * (i + 2)); a2 = __ldg(a32 + st * (i + 2)); }
                if (i + 1 < ce) b1 = load_bnd32<kRec>(P, j1);
                int sides = i < ce ? candidate_sides32(ws.rc[rl], a, b) : 0;
                if (sides & 4) {
                    const double2 bd = load_bnd(P, j);
                    sides = candidate_sides(ws.rc[rl], __ldg(val + st * i), bd.x, bd.y);
                }
                queue_push(Q, lane, sides, j, ((unsigned)i << 6) | ((unsigned)lane << 1));
                queue_drain(Q, lane, false, run);
            }
        }
        queue_drain(Q, lane, true, run);
        if (lane == 0) ws.st_div += (unsigned long long)Q.pushed;
    }
    timer_pass(lane, lg, t_pass0, t_pass1);
    report_tight(tight, lane, change, tight_ctr);
}

// One SELL-g slice per warp: 32/g rows, g lanes per row. Lane l serves row
// l >> lg and its elements sub, sub+g, ... (sub = l & (g-1)), stored
// column-major (step i of lane l at slice_ptr[slice] + 32 i + l).
// The FP32 screen runs here; rows it cannot skip take the exact pass in place
// or, with P.defer_exact, are queued for the exact-rows phase.
template <int kRec>
__device__ __forceinline__ void sell_slice(const DevProblem &P, int slice, int lane, int round, bool marked,
                                           int *change, unsigned *tight_ctr, WarpSmem &ws, int par = 0) {
    const int lg = __ldg(P.slice_lg + slice);
    const int g = 1 << lg;
    const int row0 = __ldg(P.slice_row0 + slice);
    const int nrows = __ldg(P.slice_row0 + slice + 1) - row0;
    const int rl = lane >> lg, sub = lane & (g - 1);
    const int r = row0 + rl;
    bool act = rl < nrows;
    if (act && marked) act = P.mark[r] == round;
    if (!__any_sync(kFull, act)) return;
    const int len = act ? __ldg(P.srow_len + r) : 0;
    const int cnt = len > sub ? (len - sub + g - 1) >> lg : 0;  // my elements
    const long long base = __ldg(P.slice_ptr + slice) + lane;
    const bool leader = act && sub == 0;
    const int xbase = (leader && P.defer_exact) ? __ldg(P.xptr + r) : 0;  // used at the end

    // FP32 screen
    bool exact = false;
    double lhs = 0.0, rhs = 0.0;
    float slack_lo = 0.0f;  // the screen's lower bound of its slacks, leaders of exact rows
    {
        const int *col = P.sell_col + base;
        const float *val = P.sell_a32 + base;
        Scr c;
        scr_init(c);
        int chg = 0;
#pragma unroll 4
        for (int i = 0; i < cnt; i++) {
            const int j = __ldcs(col + 32 * i);
            const float a = __ldcs(val + 32 * i);
            scr_add(c, a, load_bnd32_chg<kRec>(P, j, round, chg));
        }
        if (g > 1) {
            scr_group_reduce(c, g);
            for (int off = g >> 1; off > 0; off >>= 1) chg |= __shfl_xor_sync(kFull, chg, off);
        }
        if (leader) {
            lhs = __ldg(P.srow_lhs + r);
            rhs = __ldg(P.srow_rhs + r);
            exact = !scr_skips(c, len, lhs, rhs) && row_due<kRec>(P, round, chg);
            if (exact) {
                float hi;
                scr_slack(c, len, lhs, rhs, slack_lo, hi);
            }
        }
    }
    count_work(ws, lane, leader ? 1 : 0, leader ? len : 0, (leader && exact) ? len : 0);
    if (P.defer_exact) {
        const unsigned bal = __ballot_sync(kFull, exact);
        if (!bal) return;
        unsigned first = 0;
        if (lane == 0) first = atomicAdd(P.xctr + 16 * par + lg, (unsigned)__popc(bal));
        first = __shfl_sync(kFull, first, 0);
        if (exact) P.xrow[P.cls_begin[lg] + first + __popc(bal & ((1u << lane) - 1u))] = XRow{xbase, r, len, slack_lo, 0};
        return;
    }
    exact = __shfl_sync(kFull, exact, rl << lg) && act;
    if (!__any_sync(kFull, exact)) return;
    ws.base[lane] = base;
    __syncwarp();
    sell_rows_exact<kRec>(P, sell_view(P), lg, lane, exact, len, cnt, lhs, rhs, r, slack_lo, change, tight_ctr, ws);
}

// K slices of one-lane rows (g = 1) screened together in the deferred-exact
// mode: lane l screens row l of each slice, so the K rows' column, coefficient
// and bound loads are in flight at the same time (a slice of short rows holds
// only 64..128 non-zeros: alone, its chain of dependent loads leaves the warp
// waiting), and the exact rows of all K slices are queued with one counter
// update. Decisions and queue contents equal those of K sell_slice calls.
constexpr int kScreenGroup = 2;
template <int K, int kRec>
__device__ __forceinline__ void sell_slices_g1(const DevProblem &P, const int (&sl)[K], int lane, int round,
                                               bool marked, WarpSmem &ws, int par) {
    int r[K], len[K];
    long long base[K];
    double lhs[K], rhs[K];
    bool act[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int row0 = __ldg(P.slice_row0 + sl[k]);
        r[k] = row0 + lane;
        act[k] = lane < __ldg(P.slice_row0 + sl[k] + 1) - row0;
        base[k] = __ldg(P.slice_ptr + sl[k]) + lane;
    }
    if (marked) {
#pragma unroll
        for (int k = 0; k < K; k++)
            if (act[k]) act[k] = P.mark[r[k]] == round;
    }
    int mx = 0, xbase[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        len[k] = act[k] ? __ldg(P.srow_len + r[k]) : 0;
        xbase[k] = act[k] ? __ldg(P.xptr + r[k]) : 0;
        mx = max(mx, len[k]);
    }
    Scr c[K];
    int chg[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        scr_init(c[k]);
        chg[k] = 0;
    }
#pragma unroll 2
    for (int i = 0; i < mx; i++) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (i < len[k]) {
                const int j = __ldcs(P.sell_col + base[k] + 32 * i);
                const float a = __ldcs(P.sell_a32 + base[k] + 32 * i);
                scr_add(c[k], a, load_bnd32_chg<kRec>(P, j, round, chg[k]));
            }
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        lhs[k] = 0.0;
        rhs[k] = 0.0;
        if (act[k]) {
            lhs[k] = __ldg(P.srow_lhs + r[k]);
            rhs[k] = __ldg(P.srow_rhs + r[k]);
        }
    }
    bool exact[K];
    float slo[K];
    int rows = 0, nnz = 0, nnz_exact = 0, total = 0;
    unsigned bal[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        exact[k] = act[k] && !scr_skips(c[k], len[k], lhs[k], rhs[k]) && row_due<kRec>(P, round, chg[k]);
        slo[k] = 0.0f;
        if (exact[k]) {
            float hi;
            scr_slack(c[k], len[k], lhs[k], rhs[k], slo[k], hi);
        }
        rows += act[k] ? 1 : 0;
        nnz += len[k];
        nnz_exact += exact[k] ? len[k] : 0;
        bal[k] = __ballot_sync(kFull, exact[k]);
        total += __popc(bal[k]);
    }
    count_work(ws, lane, rows, nnz, nnz_exact);
    if (!total) return;
    unsigned first = 0;
    if (lane == 0) first = atomicAdd(P.xctr + 16 * par, (unsigned)total);
    first = __shfl_sync(kFull, first, 0) + (unsigned)P.cls_begin[0];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < K; k++) {
        if (exact[k]) P.xrow[first + __popc(bal[k] & lt)] = XRow{xbase[k], r[k], len[k], slo[k], 0};
        first += __popc(bal[k]);
    }
}

// Exact-rows phase: the rows the screen queued, class by class (widest rows
// first), 32/g rows per warp with their elements read from the row-contiguous copy.
__device__ __forceinline__ void exact_rows_phase(const DevProblem &P, int par, int *change, unsigned *tight_ctr,
                                                 WarpSmem &ws, int lane) {
    stats_zero(ws, lane);
    for (int lg = 5; lg >= 0; lg--) {
        const int n = (int)*((volatile unsigned *)(P.xctr + 16 * par + lg));
        if (!n) continue;
        const int g = 1 << lg, per = 32 >> lg;
        const int rl = lane >> lg, sub = lane & (g - 1);
        for (;;) {
            // claims only grow: a class already claimed to its end is left
            // without an atomic (every warp of the grid passes each class)
            unsigned k0 = 0;
            if (lane == 0) {
                k0 = *((volatile unsigned *)(P.xctr + 16 * par + 8 + lg));
                if (k0 < (unsigned)n) k0 = atomicAdd(P.xctr + 16 * par + 8 + lg, (unsigned)per);
            }
            const int k = (int)__shfl_sync(kFull, k0, 0) + rl;
            if (k - rl >= n) break;
            const bool exact = k < n;
            int len = 0, cnt = 0, pos = 0;
            long long base = 0;
            double lhs = 0.0, rhs = 0.0;
            float slack_lo = 0.0f;
            if (exact) {
                const XRow x = P.xrow[P.cls_begin[lg] + k];
                const int p = x.pos;
                pos = p;
                base = x.base + sub;
                len = x.len;
                slack_lo = x.slack_lo;
                cnt = len > sub ? (len - sub + g - 1) >> lg : 0;
                if (sub == 0) {
                    lhs = __ldg(P.srow_lhs + p);
                    rhs = __ldg(P.srow_rhs + p);
                }
            }
            ws.base[lane] = base;
            __syncwarp();
            sell_rows_exact<1>(P, ElemView{P.xcol, P.xval, P.xa32, g}, lg, lane, exact, len, cnt, lhs, rhs, pos,
                            slack_lo, change, tight_ctr, ws);
            __syncwarp();
        }
    }
    stats_flush(P, ws, lane);
}

// ---- split rows: one warp per tile ----------------------------------------
// Drift bound (single-problem plain rounds; marked rounds use it): a split row
// the screen skipped with certified margin m (scr_margin) stays skippable while
// the bound D of how far its slack has fallen since -- finalize adds |a|
// (lb' - lb + ub - ub') rounded up for every tightening of one of its
// variables, infinite when an infinite bound becomes finite -- satisfies
// D (1 + 2^-22) <= m: the factor covers D's own rounding (an FP64 sum of
// rounded-up terms, up to 2^28 of them) and |a| against its FP32 copy. Such a
// row tightens nothing and is feasible, exactly as its screen would decide.
// Its work is counted as screened, so the statistics equal a full screen's.
template <int kRec>
__device__ __forceinline__ bool drift_active(const DevProblem &P) {
    return kRec != 0 && P.learned == 0 && P.lrow_margin != nullptr;
}
__device__ __forceinline__ bool drift_skips(const DevProblem &P, int row) {
    const double m = P.lrow_margin[row];
    if (!(m >= 0.0)) return false;
    return __dmul_ru(P.lrow_drift[row], 1.0 + 0x1p-22) <= m;  // false for NaN and inf drifts
}
// A screen of split row `row` refreshes its certificate (one writer per row).
__device__ __forceinline__ void drift_reset(const DevProblem &P, int row, const Scr &c, int n, double lhs,
                                            double rhs) {
    P.lrow_margin[row] = scr_margin(c, n, lhs, rhs);
    P.lrow_drift[row] = 0.0;
}
__device__ __forceinline__ void acc_shfl_reduce(Acc &s) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Acc o;
        o.minact = __shfl_down_sync(kFull, s.minact, off);
        o.maxact = __shfl_down_sync(kFull, s.maxact, off);
        o.minf = __shfl_down_sync(kFull, s.minf, off);
        o.maxf = __shfl_down_sync(kFull, s.maxf, off);
        o.km = __shfl_down_sync(kFull, s.km, off);
        o.p = __shfl_down_sync(kFull, s.p, off);
        acc_combine(s, o);
    }
}

// The reference's row test (row_go_from_max, seq_eps_max where it cannot
// decide) and the candidates of split row `row` over the element range
// [b, e) of one tile, from the row's complete activities and first maximum
// held by lane 0; the warp queues the divisions. The row's first tile also
// checks it for row-side infeasibility.
template <int kRec>
__device__ __forceinline__ void split_row_candidates(const DevProblem &P, int row, int b, int e, const Acc &s0,
                                                     int lane, int *change, unsigned *tight_ctr, WarpSmem &ws) {
    RowC c;
    int go = 0;
    double mn = 0.0;
    const int t0 = __ldg(P.lrow_tile0 + row);
    const int rb = __ldg(P.tile_begin + t0);
    if (lane == 0) {
        const double lhs = __ldg(P.lrow_lhs + row), rhs = __ldg(P.lrow_rhs + row);
        mn = row_min_slack(s0.minact, s0.maxact, lhs, rhs);
        go = row_go_from_max(s0.minf, s0.maxf, acc_max(s0), mn);
        if (b == rb && row_infeasible(s0.minact, s0.maxact, s0.minf, s0.maxf, lhs, rhs))
            record_row_infeasible(P, P.n_srows + row);
        c = make_rowc(s0.minact, s0.maxact, s0.minf, s0.maxf, lhs, rhs);
    }
    go = __shfl_sync(kFull, go, 0);
    if (go == 2) {  // every tile of the row reaches the same m
        const int re = __ldg(P.tile_end + __ldg(P.lrow_tile0 + row + 1) - 1);
        const double m = seq_eps_max(P, P.lcol + rb, P.lval + rb, re - rb, __shfl_sync(kFull, s0.km, 0),
                                     __shfl_sync(kFull, s0.p, 0), lane);
        if (lane == 0) {
            go = eps_le(m, mn) ? 0 : 1;
            if (b == rb) ws.st_seq++;
        }
        go = __shfl_sync(kFull, go, 0);
    }
    if (!go) return;
    c.slack = __shfl_sync(kFull, c.slack, 0);
    c.surplus = __shfl_sync(kFull, c.surplus, 0);
    c.neg_surplus = __shfl_sync(kFull, c.neg_surplus, 0);
    c.minf = __shfl_sync(kFull, c.minf, 0);
    c.maxf = __shfl_sync(kFull, c.maxf, 0);
    c.ok = __shfl_sync(kFull, c.ok, 0);
    c.slack_dn = __shfl_sync(kFull, c.slack_dn, 0);
    c.slack_hi = __shfl_sync(kFull, c.slack_hi, 0);
    c.nsur_dn = __shfl_sync(kFull, c.nsur_dn, 0);
    c.nsur_hi = __shfl_sync(kFull, c.nsur_hi, 0);
    int tight = 0;
    WarpQueue Q{ws.q, 0, 0};
    auto run = [&](const QEntry &q) {
        const double a = __ldg(P.lval + b + (int)(q.code >> 1));
        tight += apply_side(P, c, q.j, a, load_bnd(P, q.j), (int)(q.code & 1u)) ? 1 : 0;
    };
    // software pipeline as in sell_rows_exact: two steps of columns and
    // coefficients, one step of bounds ahead
    int j1 = 0, j2 = 0;
    float a1 = 0.0f, a2 = 0.0f;
    float2 b1 = make_float2(0.0f, 0.0f);
    if (b + lane < e) { j1 = __ldg(P.lcol + b + lane); a1 = __ldg(P.la32 + b + lane); }
    if (b + 32 + lane < e) { j2 = __ldg(P.lcol + b + 32 + lane); a2 = __ldg(P.la32 + b + 32 + lane); }
    if (b + lane < e) b1 = load_bnd32<kRec>(P, j1);
    for (int k0 = b; k0 < e; k0 += 32) {
        const int k = k0 + lane;
        const int j = j1;
        const float a = a1;
        const float2 bb = b1;
        j1 = j2;
        a1 = a2;
        if (k + 64 < e) { j2 = __ldg(P.lcol + k + 64); a2 = __ldg(P.la32 + k + 64); }
        if (k + 32 < e) b1 = load_bnd32<kRec>(P, j1);
        int sides = k < e ? candidate_sides32(c, a, bb) : 0;
        if (sides & 4) {
            const double2 bd = load_bnd(P, j);
            sides = candidate_sides(c, __ldg(P.lval + k), bd.x, bd.y);
        }
        queue_push(Q, lane, sides, j, (unsigned)(k - b) << 1);
        queue_drain(Q, lane, false, run);
    }
    queue_drain(Q, lane, true, run);
    if (lane == 0) ws.st_div += (unsigned long long)Q.pushed;
    report_tight(tight, lane, change, tight_ctr);
}

__device__ __forceinline__ void scr_shfl_reduce(Scr &c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Scr o;
        o.mn = __shfl_down_sync(kFull, c.mn, off);
        o.mx = __shfl_down_sync(kFull, c.mx, off);
        o.S = __shfl_down_sync(kFull, c.S, off);
        o.U = __shfl_down_sync(kFull, c.U, off);
        o.minf = __shfl_down_sync(kFull, c.minf, off);
        o.maxf = __shfl_down_sync(kFull, c.maxf, off);
        scr_combine(c, o);
    }
}

// Exact FP64 partial of the element range [b, e) of a split row whose first
// element is rb: lane l sums elements l, l+32, ... in order, shuffle tree
// across lanes, with the first maximum of |a| (ub - lb) (indices from rb);
// lane 0 holds the result.
__device__ __forceinline__ Acc tile_exact(const DevProblem &P, int b, int e, int rb, int lane) {
    Acc s;
    acc_init(s);
#pragma unroll 4
    for (int k = b + lane; k < e; k += 32) {
        const int j = __ldg(P.lcol + k);
        const double a = __ldg(P.lval + k);
        const double2 bb = load_bnd(P, j);
        acc_add_terms(s, a, bb.x, bb.y);
        acc_add_delta(s, dmul(fabs(a), dsub(bb.y, bb.x)), k - rb);
    }
    acc_shfl_reduce(s);
    return s;
}

// Activity phase, split-row tile t: the FP32 screen of the tile. A row that
// fits in one tile is finished here (screen decision, exact pass, candidates);
// tiles of longer rows store their screen partial for the candidate phase
// (returns true for those).
template <int kRec>
__device__ __forceinline__ bool split_partial(const DevProblem &P, int t, int lane, int round, bool marked,
                                              int *change, unsigned *tight_ctr, WarpSmem &ws) {
    const int row = __ldg(P.tile_row + t);
    if (marked && P.mark[P.n_srows + row] != round) return false;
    const int b = __ldg(P.tile_begin + t), e = __ldg(P.tile_end + t);
    const int t0 = __ldg(P.lrow_tile0 + row);
    const bool single = __ldg(P.lrow_tile0 + row + 1) - t0 == 1;
    if (marked && drift_active<kRec>(P) && drift_skips(P, row)) {  // the same values for every lane
        if (lane == 0) {
            ws.st_nnz += (unsigned long long)(e - b);
            ws.st_drift_nnz += (unsigned long long)(e - b);
            if (t == t0) {
                ws.st_rows += 1ULL;
                ws.st_drift += 1ULL;
            }
            if (!single) P.lrow_skip[row] = round;  // the candidate phase skips the row too
        }
        return false;
    }
    Scr c;
    scr_init(c);
    int chg = 0;
#pragma unroll 4
    for (int k = b + lane; k < e; k += 32) {
        const int j = __ldcs(P.lcol + k);
        const float a = __ldcs(P.la32 + k);
        scr_add(c, a, load_bnd32_chg<kRec>(P, j, round, chg));
    }
    scr_shfl_reduce(c);
    chg = __any_sync(kFull, chg) ? 1 : 0;
    int exact = 0;
    if (lane == 0) {
        ws.st_nnz += (unsigned long long)(e - b);
        if (t == t0) ws.st_rows += 1ULL;
        if (single) {
            const double lhs = __ldg(P.lrow_lhs + row), rhs = __ldg(P.lrow_rhs + row);
            exact = !scr_skips(c, e - b, lhs, rhs) && row_due<kRec>(P, round, chg);
            if (drift_active<kRec>(P)) drift_reset(P, row, c, e - b, lhs, rhs);
            if (exact) ws.st_exact += (unsigned long long)(e - b);
        } else {
            TileScr ts;
            ts.mn = c.mn; ts.mx = c.mx; ts.S = c.S; ts.U = c.U; ts.minf = c.minf; ts.maxf = c.maxf;
            ts.chg = chg;
            ts.pad = 0;
            P.tile_scr[t] = ts;
        }
    }
    if (!single) return true;
    if (!__shfl_sync(kFull, exact, 0)) return false;
    const Acc s = tile_exact(P, b, e, b, lane);
    split_row_candidates<kRec>(P, row, b, e, s, lane, change, tight_ctr, ws);
    return false;
}

// Candidate phase, tile t of a multi-tile row: the row's screen (the tile
// partials combined by all lanes in a fixed order, so every tile of the row
// reaches the same decision); a row the screen cannot skip gets this tile's
// exact FP64 partial, and its first tile flags the row for the exact phase
// (returns true when the tile computed its exact partial).
template <int kRec>
__device__ __forceinline__ bool split_cand(const DevProblem &P, int t, int lane, int round, bool marked,
                                           int *exact_ctr, WarpSmem &ws) {
    const int row = __ldg(P.tile_row + t);
    if (marked && P.mark[P.n_srows + row] != round) return false;
    if (drift_active<kRec>(P) && P.lrow_skip[row] == round) return false;  // skipped on its drift bound
    const int t0 = __ldg(P.lrow_tile0 + row), t1 = __ldg(P.lrow_tile0 + row + 1);
    Scr c;
    scr_init(c);
    int chg = 0;
    for (int u = t0 + lane; u < t1; u += 32) {
        const TileScr p = P.tile_scr[u];
        Scr o;
        o.mn = p.mn; o.mx = p.mx; o.S = p.S; o.U = p.U; o.minf = p.minf; o.maxf = p.maxf;
        scr_combine(c, o);
        chg |= p.chg;
    }
    scr_shfl_reduce(c);
    chg = __any_sync(kFull, chg) ? 1 : 0;
    int exact = 0;
    if (lane == 0) {
        const int n_row = __ldg(P.tile_end + t1 - 1) - __ldg(P.tile_begin + t0);
        const double lhs = __ldg(P.lrow_lhs + row), rhs = __ldg(P.lrow_rhs + row);
        exact = !scr_skips(c, n_row, lhs, rhs) && row_due<kRec>(P, round, chg);
        if (drift_active<kRec>(P) && t == t0) drift_reset(P, row, c, n_row, lhs, rhs);
    }
    if (!__shfl_sync(kFull, exact, 0)) return false;
    const int b = __ldg(P.tile_begin + t), e = __ldg(P.tile_end + t);
    const Acc s = tile_exact(P, b, e, __ldg(P.tile_begin + t0), lane);
    if (lane == 0) {
        TilePart tp;
        tp.minact = s.minact; tp.maxact = s.maxact; tp.km = s.km; tp.minf = s.minf; tp.maxf = s.maxf;
        tp.p = s.p;
        tp.pad = 0;
        P.tile_part[t] = tp;
        ws.st_exact += (unsigned long long)(e - b);
        if (t == t0) {
            P.row_exact[row] = round;
            atomicAdd(exact_ctr, 1);
        }
    }
    return true;
}

// Exact phase, tile t of a multi-tile row flagged this round: the row's exact
// partials combined in tile order, then the decision and this tile's candidates.
template <int kRec>
__device__ __forceinline__ void split_exact(const DevProblem &P, int t, int lane, int round, int *change,
                                            unsigned *tight_ctr, WarpSmem &ws, int part = 0, int parts = 1) {
    const int row = __ldg(P.tile_row + t);
    if (P.row_exact[row] != round) return;
    // lanes load 32 partials at a time; lane 0 folds them in tile order
    const int t0 = __ldg(P.lrow_tile0 + row), t1 = __ldg(P.lrow_tile0 + row + 1);
    Acc s;
    acc_init(s);
    for (int b = t0; b < t1; b += 32) {
        TilePart tp = {0.0, 0.0, 0, 0, 0, -1, 0};
        if (b + lane < t1) tp = P.tile_part[b + lane];
        const int cnt = min(32, t1 - b);
        for (int i = 0; i < cnt; i++) {
            Acc o;
            o.minact = __shfl_sync(kFull, tp.minact, i);
            o.maxact = __shfl_sync(kFull, tp.maxact, i);
            o.minf = __shfl_sync(kFull, tp.minf, i);
            o.maxf = __shfl_sync(kFull, tp.maxf, i);
            o.km = __shfl_sync(kFull, tp.km, i);
            o.p = __shfl_sync(kFull, tp.p, i);
            if (lane == 0) {
                if (b + i == t0) s = o;
                else acc_combine(s, o);
            }
        }
    }
    // this item's part of the tile: parts of whole warp steps
    const int tb = __ldg(P.tile_begin + t), te = __ldg(P.tile_end + t);
    const int step = ((te - tb + parts - 1) / parts + 31) & ~31;
    const int pb = min(te, tb + part * step), pe = min(te, pb + step);
    if (pb < pe) split_row_candidates<kRec>(P, row, pb, pe, s, lane, change, tight_ctr, ws);
}

// Adds a thread's committed-change count to the round flags, one atomic per warp.
__device__ __forceinline__ void flush_changed(const DevProblem &P, unsigned long long changed) {
    const unsigned active = __activemask();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) changed += __shfl_down_sync(active, changed, off);
    if ((threadIdx.x & 31) == __ffs(active) - 1 && changed) atomicAdd(&P.flags[0].changed_vars, changed);
}

// Commit changed variables nxt -> cur, apply the infeasibility rules (a row
// recorded infeasible in this round, a variable whose bounds cross), mark the
// rows of changed variables for the next round, clear the bitmap.
// One warp per word of the bitmap: lane l commits variable 32 w + l, then the
// warp pushes the marks of each changed variable's rows together, 32 per step
// (a thread walking its word's variables and their rows alone leaves the
// commit of a round with many changes to a few long serial chains). tid /
// nthreads: a grid of whole warps.
__device__ __forceinline__ void finalize_words(const DevProblem &P, int round, bool push_marks, int tid,
                                               int nthreads) {
    const int lane = tid & 31;
    unsigned long long changed = 0;
    if (tid == 0 && P.flags[0].infeasible_row != INT_MAX) P.flags[0].infeasible = 1;
    for (int w = tid >> 5; w < P.n_chg_words; w += nthreads >> 5) {
        const unsigned bits = P.chg[w];
        if (!bits) continue;  // warp-uniform
        double delta = 0.0;  // upper bound of (lb' - lb) + (ub - ub') of my variable
        if ((bits >> lane) & 1u) {
            const int j = w * 32 + lane;
            const double2 b = P.bnd_nxt[j];
            const double2 o = P.bnd[j];
            delta = (neginf_bits(dbits(o.x)) || posinf_bits(dbits(o.y)))
                            ? __longlong_as_double(0x7FF0000000000000LL)  // an infinite bound became finite
                            : __dadd_ru(__dsub_ru(b.x, o.x), __dsub_ru(o.y, b.y));
            P.bnd[j] = b;
            store_bnd32<1>(P, j, b, round);
            if (var_infeasible(b.x, b.y)) {
                P.flags[0].infeasible = 1;
                atomicMin(&P.flags[0].infeasible_var, j);
            }
        }
        __syncwarp();
        if (lane == 0) {
            P.chg[w] = 0u;
            changed += __popc(bits);
        }
        if (!push_marks) continue;
        for (unsigned rem = bits; rem; rem &= rem - 1) {
            const int bit = __ffs(rem) - 1;
            const int j = w * 32 + bit;
            const double dj = __shfl_sync(kFull, delta, bit);
            for (int p = __ldg(P.var_ptr + j) + lane; p < __ldg(P.var_ptr + j + 1); p += 32) {
                const int2 e = __ldg(reinterpret_cast<const int2 *>(P.var_ent) + p);  // {pos, acoef}
                const int pos = e.x;
                P.mark[pos] = round + 1;
                // a split row's slack moves by at most |a| (lb' - lb + ub - ub')
                if (pos >= P.n_srows && P.lrow_drift)
                    atomicAdd(P.lrow_drift + (pos - P.n_srows), __dmul_ru((double)__int_as_float(e.y), dj));
            }
        }
    }
    flush_changed(P, changed);
}

// ---- work distribution ----------------------------------------------------
// Warp-level dynamic queue over items sorted heaviest first.
__device__ __forceinline__ int warp_next(unsigned *ctr, int lane) {
    unsigned v = 0;
    if (lane == 0) v = atomicAdd(ctr, 1u);
    return (int)__shfl_sync(kFull, v, 0);
}

__device__ __forceinline__ void activity_item(const DevProblem &P, int it, int lane, int round, bool marked,
                                              int *change, unsigned *tight_ctr, WarpSmem &ws, int par) {
    if (it >= 0) sell_slice<1>(P, it, lane, round, marked, change, tight_ctr, ws, par);
    else split_partial<1>(P, -it - 1, lane, round, marked, change, tight_ctr, ws);
}

// Items are claimed kScreenGroup at a time; a claim of one-lane-row slices
// (the light end of the heaviest-first order) is screened as a group when
// exact rows are deferred, other claims item by item.
__device__ __forceinline__ void activity_phase(const DevProblem &P, int round, bool marked, unsigned *ctr,
                                               int *change, unsigned *tight_ctr, WarpSmem &ws, int lane,
                                               int par = 0) {
    stats_zero(ws, lane);
    constexpr int K = kScreenGroup;
    WarpCursor cur;
    cur.start(ctr, (unsigned)K, lane);
    for (;;) {
        const int i = cur.next(lane);
        if (i >= P.n_items) break;
        int it[K];
        bool group = P.defer_exact && i + K <= P.n_items;
#pragma unroll
        for (int k = 0; k < K; k++) {
            it[k] = i + k < P.n_items ? __ldg(P.items + i + k) : -1;
            group = group && it[k] >= 0;
        }
        if (group) {
#pragma unroll
            for (int k = 0; k < K; k++) group = group && __ldg(P.slice_lg + it[k]) == 0;
        }
        if (group) {
            sell_slices_g1<K, 1>(P, it, lane, round, marked, ws, par);
        } else {
#pragma unroll 1
            for (int k = 0; k < K && i + k < P.n_items; k++)
                activity_item(P, it[k], lane, round, marked, change, tight_ctr, ws, par);
        }
    }
    stats_flush(P, ws, lane);
}

// The grid's warps: this warp's index and their number.
__device__ __forceinline__ int grid_warp() { return (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); }
__device__ __forceinline__ int grid_warps() { return (int)((gridDim.x * blockDim.x) >> 5); }

// Candidate phase over the tiles of multi-tile rows: warp w takes the tiles
// w, w + W, ... (W warps), one per lane per step, and runs those whose row is
// due (every tile in an unmarked round, the tiles of marked rows otherwise).
// The tiles hold at most split_tile non-zeros each and the deferred exact rows
// that follow in the same phase are claimed dynamically, so a static
// assignment costs no balance and saves a contended claim per tile.
__device__ __forceinline__ void candidate_phase(const DevProblem &P, int round, bool marked, unsigned *ctr,
                                                int *exact_ctr, WarpSmem &ws, int lane) {
    (void)ctr;
    stats_zero(ws, lane);
    const int nw = grid_warps();
    for (int i0 = grid_warp(); i0 < P.n_mtiles; i0 += 32 * nw) {
        const int i = i0 + lane * nw;
        int t = 0;
        bool live = false;
        if (i < P.n_mtiles) {
            t = __ldg(P.mtiles + i);
            live = !marked || P.mark[P.n_srows + __ldg(P.tile_row + t)] == round;
        }
        for (unsigned bal = __ballot_sync(kFull, live); bal; bal &= bal - 1)
            split_cand<1>(P, __shfl_sync(kFull, t, __ffs(bal) - 1), lane, round, false, exact_ctr, ws);
    }
    stats_flush(P, ws, lane);
}

// Exact phase over the tiles of the multi-tile rows flagged this round, with
// the same static assignment as the candidate phase, each tile's candidates in
// quarters (a warp per quarter): the row test is the same for every quarter,
// and a tile's 1,024 candidate tests and divisions on one warp were the
// phase's long pole while the rest of the grid waited at its barrier.
__device__ __forceinline__ void exact_phase(const DevProblem &P, int round, unsigned *ctr, int *change,
                                            unsigned *tight_ctr, WarpSmem &ws, int lane) {
    (void)ctr;
    stats_zero(ws, lane);
    constexpr int kParts = 4;  // candidates of a tile in quarters: a long tile is no phase's long pole
    const int nw = grid_warps();
    const int n_items = P.n_mtiles * kParts;
    for (int i0 = grid_warp(); i0 < n_items; i0 += 32 * nw) {
        const int i = i0 + lane * nw;
        int t = 0;
        bool live = false;
        if (i < n_items) {
            t = __ldg(P.mtiles + i / kParts);
            live = P.row_exact[__ldg(P.tile_row + t)] == round;
        }
        for (unsigned bal = __ballot_sync(kFull, live); bal; bal &= bal - 1) {
            const int src = __ffs(bal) - 1;
            split_exact<1>(P, __shfl_sync(kFull, t, src), lane, round, change, tight_ctr, ws,
                           (i0 + src * nw) % kParts, kParts);
        }
    }
    stats_flush(P, ws, lane);
}

// Whether the activity phase of this round's parity queued exact rows.
__device__ __forceinline__ bool exact_rows_queued(const DevProblem &P, int par) {
    if (!P.defer_exact) return false;
    unsigned n = 0;
#pragma unroll
    for (int lg = 0; lg < 6; lg++) n |= *((volatile unsigned *)(P.xctr + 16 * par + lg));
    return n != 0;
}

// Whether the round after one with `tight` tightenings runs on marked rows.
__device__ __forceinline__ bool next_round_marked(const DevProblem &P, unsigned tight) {
    return P.use_marking == 2 || (P.use_marking == 1 && tight < P.mark_threshold);
}

// Grid barrier with a bounded wait: thread 0 of each CTA reads the barrier
// generation, arrives, and spins until the generation moves. Any CTA that
// waits longer than `limit` clock64 cycles (or sees another CTA's error)
// records kErrBarrierTimeout and every CTA leaves the round loop at its next
// barrier. The default limit is 4e9 cycles, about 2 s at 2 GHz.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *error, long long limit) {
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = bar + 1;
        const unsigned my_gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == my_gen) {
                if (*((volatile int *)error) != kErrNone) { ok = 0; break; }
                if (clock64() - t0 > limit) {
                    atomicExch(error, (int)kErrBarrierTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*((volatile int *)error) != kErrNone) ok = 0;
    }
    return __syncthreads_and(ok) != 0;
}

}  // namespace
}  // namespace gdp

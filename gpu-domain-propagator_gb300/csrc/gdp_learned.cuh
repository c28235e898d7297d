// gdp_learned.cuh -- device code of learned row marking shared by the
// single-problem learned loop (gdp_learned.cu) and the batched engine
// (gdp_batch.cu): row features, the learned slice step and the rule that
// picks the next round's kind.
#pragma once

#include "gdp_round.cuh"

namespace gdp {
namespace {

constexpr int kRowInfoStreakShift = 8;
constexpr int kMaxDeferRounds = 4;  // a marked row waits at most this many rounds for processing

// The 16 features of row position p before it is processed in `round`.
__device__ __forceinline__ void row_features(const DevProblem &P, int p, int round, int len, double lhs,
                                             double rhs, float (&v)[16]) {
    const int lp = P.last_proc[p], lt = P.last_tight[p], dr = P.dirty[p], dc = P.dcount[p];
    const unsigned info = P.rinfo[p];
    const float2 st = P.rstat[p];
    v[0] = log2f(1.f + (float)len) * (1.f / 16.f);
    v[1] = (float)(info & 3u) * (1.f / 3.f);
    v[2] = (float)((info >> 2) & 3u) * (1.f / 3.f);
    v[3] = st.x;
    v[4] = st.y;
    v[5] = neginf_bits(dbits(lhs)) ? 1.f : 0.f;
    v[6] = posinf_bits(dbits(rhs)) ? 1.f : 0.f;
    v[7] = dbits(lhs) == dbits(rhs) ? 1.f : 0.f;
    v[8] = (float)(lt ? min(round - lt, 63) : 63) * (1.f / 63.f);
    v[9] = (float)(lp ? min(round - lp, 63) : 63) * (1.f / 63.f);
    v[10] = (float)(dr ? min(round - dr, 63) : 0) * (1.f / 63.f);
    v[11] = fminf((float)dc / (float)max(len, 1), 1.f);
    v[12] = fminf((float)((info >> kRowInfoStreakShift) & 255u) * (1.f / 15.f), 1.f);
    v[13] = (float)((info >> 4) & 1u);
    v[14] = (float)((info >> 5) & 1u);
    v[15] = lp == 0 ? 1.f : 0.f;
}

// Screen statistics kept for the row's next features.
__device__ __forceinline__ float2 screen_stats(const Scr &c, int n, double lhs, double rhs) {
    float mn_lo, mn_hi;
    scr_slack(c, n, lhs, rhs, mn_lo, mn_hi);
    float2 r;
    if (!(mn_hi < kInfF32Dn) || !(mn_lo > -kInfF32Dn)) {
        r.x = 1.f;
        r.y = -1.f;
        return r;
    }
    const float mid = 0.5f * (mn_lo + mn_hi);
    r.x = fminf(fmaxf(mid / (c.S + 1e-30f), -1.f), 1.f);
    r.y = fminf(fmaxf(log2f(fmaxf(c.U, 1e-30f) / fmaxf(fabsf(mid), 1e-30f)) * (1.f / 32.f), -1.f), 1.f);
    return r;
}

enum RoundKind : int { kRoundFull = 0, kRoundLearned = 1, kRoundFlush = 2 };

// One SELL-g slice in a round of the given kind. Returns true when the model
// deferred marked rows of the slice (they stay dirty for a later round).
template <int kRec>  // the bnd32 layout (load_bnd32): 1 in contexts, 0 in batch members
__device__ __forceinline__ bool sell_slice_learned(const DevProblem &P, int slice, int lane, int round, int kind,
                                                   int *change, unsigned *tight_ctr, WarpSmem &ws,
                                                   LearnSmem &L) {
    const bool full = kind == kRoundFull;
    const int lg = __ldg(P.slice_lg + slice);
    const int g = 1 << lg;
    const int row0 = __ldg(P.slice_row0 + slice);
    const int nrows = __ldg(P.slice_row0 + slice + 1) - row0;
    const int rl = lane >> lg, sub = lane & (g - 1);
    const int r = row0 + rl;
    bool act = rl < nrows && (full || P.dirty[r] != 0);
    {
        const unsigned mk = __ballot_sync(kFull, act && sub == 0);
        if (lane == 0) L.marked += __popc(mk);
    }
    if (!__any_sync(kFull, act)) return false;
    bool any_deferred = false;  // marked rows the model left for a later round
    const int len = act ? __ldg(P.srow_len + r) : 0;
    const bool leader0 = act && sub == 0;
    double lhs = 0.0, rhs = 0.0;
    if (leader0) {
        lhs = __ldg(P.srow_lhs + r);
        rhs = __ldg(P.srow_rhs + r);
    }
    // features (trace rounds: every marked row; learned rounds: the rows the
    // model decides for -- marked, at least learn_min_len long and younger
    // than the deferral cap; the others are processed whatever their score)
    const bool logged = P.learned == 2 && !full;
    const bool select = P.learned == 1 && kind == kRoundLearned;
    // a row the model can ever score: its state (features of later rounds) is kept
    const bool scored_row = P.learned == 2 || len >= P.learn_min_len;
    const bool decide = select && leader0 && scored_row && round - P.dirty[r] < kMaxDeferRounds;
    __nv_bfloat16 (*feat)[16] = reinterpret_cast<__nv_bfloat16 (*)[16]>(ws.q);
    unsigned trace_idx = 0xffffffffu;
    const bool any_decide = __any_sync(kFull, decide);  // every lane, outside any condition
    if (logged || (select && any_decide)) {
        if (logged ? leader0 : decide) {
            float v[16];
            row_features(P, r, round, len, lhs, rhs, v);
#pragma unroll
            for (int k = 0; k < 16; k++) feat[rl][k] = __float2bfloat16_rn(v[k]);
            if (logged) {  // trace rounds process every marked row: log its features now
                trace_idx = atomicAdd(P.trace_n, 1u);
                if (trace_idx < P.trace_cap) {
#pragma unroll
                    for (int k = 0; k < 16; k++)
                        P.trace_x[(size_t)trace_idx * 16 + k] = __bfloat162float(feat[rl][k]);
                }
            }
        }
        __syncwarp();
    }
    if (select) {
        // rows the model decides for: marked, at least learn_min_len long and
        // younger than the deferral cap (the others are processed whatever
        // their score); a 16-row tile without one is not scored
        const unsigned need = __ballot_sync(kFull, decide);
        const int ntiles = ((32 >> lg) + 15) >> 4;
        for (int tile = 0; tile < ntiles; tile++) {
            if (!(need & (lg == 0 ? 0xFFFFu << (16 * tile) : kFull))) continue;  // warp-uniform
            unsigned a[4];
            load_a_smem(&feat[tile * 16][0], lane, a);
            float z0, z1;
            mlp_infer_tile(P.mlp, a, lane, z0, z1);
            if ((lane & 3) == 0) {
                L.z[tile * 16 + (lane >> 2)] = z0;
                L.z[tile * 16 + (lane >> 2) + 8] = z1;
            }
        }
        __syncwarp();
        // rows shorter than the model's minimum length are always processed:
        // deferring them saves little and may stall a propagation front; a
        // row whose first unprocessed change is kMaxDeferRounds rounds old is
        // processed too, so that no row is deferred (and scored) round after
        // round while a long propagation never lets a flush happen (L.z of
        // those rows may be stale: their tile may have gone unscored)
        // every lane takes part in the shuffle (a full-mask shuffle that some
        // lanes skip is undefined), then each row keeps or defers as one
        const bool row_decided = __shfl_sync(kFull, decide, rl << lg);
        const bool keep = act && (!row_decided || L.z[rl] >= P.tau);
        const unsigned deferred = __ballot_sync(kFull, leader0 && !keep);
        if (lane == 0 && deferred) atomicAdd(&P.flags[0].rows_deferred, (unsigned long long)__popc(deferred));
        any_deferred = deferred != 0;
        act = keep;
        if (!__any_sync(kFull, act)) return any_deferred;
    }
    const bool leader = act && sub == 0;
    const int cnt = (act && len > sub) ? (len - sub + g - 1) >> lg : 0;
    const long long base = __ldg(P.slice_ptr + slice) + lane;
    if (leader) {
        L.tight[rl] = 0;
        L.go[rl] = 0;
    }
    // FP32 screen
    Scr c;
    scr_init(c);
    {
        const int *col = P.sell_col + base;
        const float *val = P.sell_a32 + base;
#pragma unroll 4
        for (int i = 0; i < cnt; i++) {
            const int j = __ldcs(col + 32 * i);
            const float a = __ldcs(val + 32 * i);
            scr_add(c, a, load_bnd32<kRec>(P, j));
        }
    }
    if (g > 1) scr_group_reduce(c, g);
    bool exact = false;
    float2 st = make_float2(0.f, 0.f);
    float slack_lo = 0.0f;
    if (leader) {
        exact = !scr_skips(c, len, lhs, rhs);
        if (scored_row) st = screen_stats(c, len, lhs, rhs);
        if (exact) {
            float hi;
            scr_slack(c, len, lhs, rhs, slack_lo, hi);
        }
    }
    count_work(ws, lane, leader ? 1 : 0, leader ? len : 0, (leader && exact) ? len : 0);
    exact = __shfl_sync(kFull, exact, rl << lg) && act;
    __syncwarp();
    if (__any_sync(kFull, exact)) {
        ws.base[lane] = base;
        __syncwarp();
        sell_rows_exact<kRec>(P, sell_view(P), lg, lane, exact, len, cnt, lhs, rhs, r, slack_lo, change, tight_ctr, ws,
                        L.tight, L.go);
    }
    __syncwarp();
    if (leader) {
        const bool tightened = L.tight[rl] > 0;
        if (logged && trace_idx < P.trace_cap) P.trace_y[trace_idx] = tightened ? 1.f : 0.f;
        if (scored_row) {  // rows the model never scores need no feature state
            const unsigned old = P.rinfo[r];
            const unsigned streak = tightened ? 0u : min(((old >> kRowInfoStreakShift) & 255u) + 1u, 255u);
            P.rinfo[r] = (unsigned)min(c.minf, 3) | ((unsigned)min(c.maxf, 3) << 2) | ((exact ? 1u : 0u) << 4) |
                         ((L.go[rl] ? 1u : 0u) << 5) | (streak << kRowInfoStreakShift);
            P.rstat[r] = st;
            P.last_proc[r] = round;
            if (tightened) P.last_tight[r] = round;
        }
        P.dirty[r] = 0;
        P.dcount[r] = 0;
    }
    return any_deferred;
}

// The kind of the round after one of kind `kind` that found `tight`
// tightenings and met `marked` marked SELL rows (n_srows rows in all). A
// round with tightenings is followed by a LEARNED round, except that a FULL
// round is followed by a FLUSH (every row was just processed, so the model's
// features tell the rows apart by nothing yet; FULL again without marking).
// A LEARNED round without tightenings is followed by a FLUSH of the rows it
// deferred, or by a FULL round when the marked rows were at least an eighth
// of all rows. FULL and FLUSH rounds without tightenings end the propagation
// (learned_certifies).
__device__ __forceinline__ int learned_next_kind(int kind, unsigned tight, unsigned long long marked, int n_srows,
                                                 int use_marking) {
    if (tight == 0)
        return kind == kRoundLearned ? (marked * 8ULL >= (unsigned long long)n_srows ? kRoundFull : kRoundFlush)
                                     : kRoundFull;
    if (use_marking == 0) return kRoundFull;
    return kind == kRoundFull ? kRoundFlush : kRoundLearned;
}

// A round certifies the fixpoint when it changed nothing and processed every
// row whose variables changed since its last processing: a FULL round, or a
// FLUSH (every marked row; split rows are processed whenever marked, and a
// SELL row stays marked until processed).
__device__ __forceinline__ bool learned_certifies(int kind, unsigned tight) {
    return tight == 0 && (kind == kRoundFull || kind == kRoundFlush);
}

// Marks row position p dirty for round `round` (a variable of it changed):
// SELL rows count the change and keep the round of their first unprocessed
// change; split rows take the plain round-stamped mark. Returns true for a
// SELL row (the caller queues its slice) and false for a split row.
__device__ __forceinline__ bool learned_mark_position(const DevProblem &P, int p, int round) {
    if (p < P.n_srows) {
        atomicAdd(P.dcount + p, 1);
        if (P.dirty[p] == 0) atomicCAS(P.dirty + p, 0, round);
        return true;
    }
    P.mark[p] = round;
    return false;
}

}  // namespace
}  // namespace gdp

// gdp_learned.cu -- learned row marking: the round loop in which the MLP of
// gdp_mlp.cuh chooses which marked rows to process, and the trace logger that
// produces its training data.
//
// Marking is exact without the model: a row is marked ("dirty") when one of
// its variables changes and stays marked until processed. Rounds come in
// three kinds:
//   LEARNED  the marked SELL rows whose score clears the threshold, and every
//            marked row shorter than learn_min_len (the rest stay marked, their
//            features ageing, so several markings of an unproductive row
//            coalesce into one later processing);
//   FLUSH    every marked row -- after a LEARNED round that changed nothing
//            and met fewer marked rows than an eighth of all rows;
//   FULL     every row -- the first round, after a FLUSH round that changed
//            nothing, and after a LEARNED round that changed nothing with
//            more marked rows than that (with use_marking == 0, every round).
// Unlike the plain adaptive schedule, a round with many tightenings is not
// followed by a full sweep: the marks are always pushed, so that rows the
// model deferred are not swept along.
// Split rows (longer than split_tile) are processed whenever marked. The plain
// full sweep is the judge: the propagation ends only when a FULL round changes
// nothing, so the result is a certified fixpoint of the same propagation
// operator whatever the model decides.
//
// Trace mode processes every marked row (exact marking) and logs, for each
// marked SELL row of a marked round, its features before processing and the
// label "processing it tightened at least one bound".
#include "gdp_learned.h"
#include "gdp_round.cuh"

namespace gdp {

namespace {

constexpr int kRowInfoStreakShift = 8;

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

// One SELL-g slice in a round of the given kind.
__device__ __forceinline__ void sell_slice_learned(const DevProblem &P, int slice, int lane, int round, int kind,
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
    if (!__any_sync(kFull, act)) return;
    const int len = act ? __ldg(P.srow_len + r) : 0;
    const bool leader0 = act && sub == 0;
    double lhs = 0.0, rhs = 0.0;
    if (leader0) {
        lhs = __ldg(P.srow_lhs + r);
        rhs = __ldg(P.srow_rhs + r);
    }
    // features (trace rounds and learned marked rounds)
    const bool logged = P.learned == 2 && !full;
    const bool select = P.learned == 1 && kind == kRoundLearned;
    __nv_bfloat16 (*feat)[16] = reinterpret_cast<__nv_bfloat16 (*)[16]>(ws.q);
    unsigned trace_idx = 0xffffffffu;
    if (logged || select) {
        if (leader0) {
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
        const int ntiles = ((32 >> lg) + 15) >> 4;
        for (int tile = 0; tile < ntiles; tile++) {
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
        // deferring them saves little and may stall a propagation front
        const bool keep = act && (len < P.learn_min_len || L.z[rl] >= P.tau);
        const unsigned deferred = __ballot_sync(kFull, leader0 && !keep);
        if (lane == 0 && deferred) atomicAdd(&P.flags[0].rows_deferred, (unsigned long long)__popc(deferred));
        act = keep;
        if (!__any_sync(kFull, act)) return;
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
            scr_add(c, a, load_bnd32(P, j));
        }
    }
    if (g > 1) scr_group_reduce(c, g);
    bool exact = false;
    float2 st = make_float2(0.f, 0.f);
    float u_hi = 0.0f;
    if (leader) {
        exact = !scr_skips(c, len, lhs, rhs);
        st = screen_stats(c, len, lhs, rhs);
        u_hi = scr_u_bound(c);
    }
    count_work(ws, lane, leader ? 1 : 0, leader ? len : 0, (leader && exact) ? len : 0);
    exact = __shfl_sync(kFull, exact, rl << lg) && act;
    __syncwarp();
    if (__any_sync(kFull, exact)) {
        ws.base[lane] = base;
        __syncwarp();
        sell_rows_exact(P, sell_view(P), lg, lane, exact, len, cnt, lhs, rhs, u_hi, change, tight_ctr, ws, L.tight,
                        L.go);
    }
    __syncwarp();
    if (leader) {
        const bool tightened = L.tight[rl] > 0;
        if (logged && trace_idx < P.trace_cap) P.trace_y[trace_idx] = tightened ? 1.f : 0.f;
        const unsigned old = P.rinfo[r];
        const unsigned streak = tightened ? 0u : min(((old >> kRowInfoStreakShift) & 255u) + 1u, 255u);
        P.rinfo[r] = (unsigned)min(c.minf, 3) | ((unsigned)min(c.maxf, 3) << 2) | ((exact ? 1u : 0u) << 4) |
                     ((L.go[rl] ? 1u : 0u) << 5) | (streak << kRowInfoStreakShift);
        P.rstat[r] = st;
        P.last_proc[r] = round;
        if (tightened) P.last_tight[r] = round;
        P.dirty[r] = 0;
        P.dcount[r] = 0;
    }
}

__device__ __forceinline__ void learned_activity_phase(const DevProblem &P, int round, int kind, unsigned *ctr,
                                                       int *change, unsigned *tight_ctr, WarpSmem &ws,
                                                       LearnSmem &L, int lane, unsigned long long *marked_ctr) {
    stats_zero(ws, lane);
    if (lane == 0) L.marked = 0;
    __syncwarp();
    WarpCursor cur;
    cur.start(ctr, 1u, lane);
    for (;;) {
        const int i = cur.next(lane);
        if (i >= P.n_items) break;
        const int it = __ldg(P.items + i);
        if (it >= 0) sell_slice_learned(P, it, lane, round, kind, change, tight_ctr, ws, L);
        else split_partial(P, -it - 1, lane, round, kind != kRoundFull, change, tight_ctr, ws);
    }
    stats_flush(P, ws, lane);
    if (lane == 0 && L.marked) atomicAdd(marked_ctr, L.marked);
}

// Commit changed variables; mark their rows for the next round: SELL rows
// become (or stay) dirty, split rows get the next round's stamp.
__device__ __forceinline__ void learned_finalize(const DevProblem &P, int round, bool push, int tid,
                                                 int nthreads) {
    unsigned long long changed = 0;
    for (int w = tid; w < P.n_chg_words; w += nthreads) {
        unsigned bits = P.chg[w];
        if (!bits) continue;
        P.chg[w] = 0u;
        changed += __popc(bits);
        while (bits) {
            const int j = w * 32 + __ffs(bits) - 1;
            bits &= bits - 1;
            const double2 b = P.bnd_nxt[j];
            P.bnd[j] = b;
            P.bnd32[j] = bnd_screen(b);
            if (var_infeasible(b.x, b.y)) {
                P.flags[0].infeasible = 1;
                atomicMin(&P.flags[0].infeasible_var, j);
            }
            if (!push) continue;
            for (int k = __ldg(P.var_ptr + j); k < __ldg(P.var_ptr + j + 1); k++) {
                const int p = __ldg(P.var_pos + k);
                if (p < P.n_srows) {
                    atomicAdd(P.dcount + p, 1);
                    if (P.dirty[p] == 0) atomicCAS(P.dirty + p, 0, round + 1);
                } else {
                    P.mark[p] = round + 1;
                }
            }
        }
    }
    flush_changed(P, changed);
}

__global__ void __launch_bounds__(kCtaThreads, 2) k_megakernel_learned(DevProblem P) {
    __shared__ WarpSmem ws[kWarpsPerCta];
    __shared__ LearnSmem ls[kWarpsPerCta];
    const int lane = threadIdx.x & 31;
    WarpSmem &mine = ws[threadIdx.x >> 5];
    LearnSmem &L = ls[threadIdx.x >> 5];
    int *err = &P.flags[0].error;
    int last_change = 0;
    int kind = kRoundFull;  // round 1 processes every row
    if (*((volatile int *)&P.flags[0].infeasible) == 0) {
        for (int round = 1; round <= P.max_rounds; round++) {
            const int par = round & 1;
            int *change = &P.flags[1 + par].change;
            unsigned *tight = &P.flags[1 + par].tight;
            int *exact = &P.flags[1 + par].exact;
            unsigned *q = P.queue + 4 * par;
            const bool full = kind == kRoundFull;
            learned_activity_phase(P, round, kind, q + 0, change, tight, mine, L, lane,
                                   &P.flags[1 + par].rows_deferred);
            if (!grid_barrier(P.barrier, err)) return;
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                P.flags[1 + (par ^ 1)].change = 0;
                P.flags[1 + (par ^ 1)].tight = 0u;
                P.flags[1 + (par ^ 1)].exact = 0;
                P.flags[1 + (par ^ 1)].rows_deferred = 0ULL;  // this kernel's per-round marked-row count
                P.queue[4 * (par ^ 1) + 0] = 0u;
                P.queue[4 * (par ^ 1) + 1] = 0u;
                P.queue[4 * (par ^ 1) + 2] = 0u;
                if (full) P.flags[0].full_rounds += 1;
            }
            if (P.n_mtiles) {
                candidate_phase(P, round, !full, q + 1, exact, mine, lane);
                if (!grid_barrier(P.barrier, err)) return;
                if (*((volatile int *)exact)) {
                    exact_phase(P, round, q + 2, change, tight, mine, lane);
                    if (!grid_barrier(P.barrier, err)) return;
                }
            }
            const unsigned t = *((volatile unsigned *)tight);
            const bool certified = full && t == 0;
            int next;
            // a LEARNED round that changed nothing is followed by a FLUSH of the
            // deferred rows -- or directly by the certifying FULL round when
            // the marked rows were at least an eighth of all rows (a full
            // sweep then costs little more than the flush, and one of the two
            // is saved when nothing is left to tighten)
            const unsigned long long marked =
                    *((volatile unsigned long long *)&P.flags[1 + par].rows_deferred);
            if (t == 0)
                next = kind == kRoundLearned ? (marked * 8ULL >= (unsigned long long)P.n_srows ? kRoundFull
                                                                                              : kRoundFlush)
                                             : kRoundFull;
            else next = P.use_marking == 0 ? kRoundFull : kRoundLearned;
            learned_finalize(P, round, !certified && next != kRoundFull && round < P.max_rounds,
                             blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
            if (blockIdx.x == 0 && threadIdx.x == 0) P.flags[0].rounds = round;
            if (!grid_barrier(P.barrier, err)) return;
            last_change = *((volatile int *)change);
            const int infeasible = *((volatile int *)&P.flags[0].infeasible);
            if (certified || infeasible) break;
            kind = next;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.flags[0].change = last_change;
        P.flags[0].done = 1;
    }
}

__global__ void __launch_bounds__(256) k_learned_reset(DevProblem P) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_srows; p += gridDim.x * blockDim.x) {
        P.dirty[p] = 0;
        P.dcount[p] = 0;
        P.last_proc[p] = 0;
        P.last_tight[p] = 0;
        P.rstat[p] = make_float2(0.f, 0.f);
        P.rinfo[p] = 0u;
    }
}

}  // namespace

int launch_learned(const DevProblem &P, int grid, int vec_blocks, cudaStream_t s) {
    k_learned_reset<<<vec_blocks, 256, 0, s>>>(P);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    DevProblem Pc = P;
    void *args[] = {&Pc};
    return (int)cudaLaunchCooperativeKernel((const void *)k_megakernel_learned, dim3(grid), dim3(kCtaThreads), args,
                                            0, s);
}

int learned_occupancy(int *blocks_per_sm) {
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_megakernel_learned, kCtaThreads, 0);
}

}  // namespace gdp

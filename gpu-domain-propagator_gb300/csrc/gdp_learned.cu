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
//   FLUSH    every marked row -- after the first round (and any FULL round)
//            that tightened, and after a LEARNED round that changed nothing
//            and met fewer marked rows than an eighth of all rows;
//   FULL     every row -- the first round, and after a LEARNED round that
//            changed nothing with more marked rows than that (with
//            use_marking == 0, every round).
// Unlike the plain adaptive schedule, a round with many tightenings is not
// followed by a full sweep: the marks are always pushed, so that rows the
// model deferred are not swept along.
// Split rows (longer than split_tile) are processed whenever marked. The
// propagation ends when a FULL or FLUSH round changes nothing: such a round
// processed every row whose variables changed since its last processing, so
// the result is a certified fixpoint of the same propagation operator
// whatever the model decides (the certificate of exact marking).
//
// Trace mode processes every marked row (exact marking) and logs, for each
// marked SELL row of a marked round, its features before processing and the
// label "processing it tightened at least one bound".
#include "gdp_learned.h"
#include "gdp_learned.cuh"

namespace gdp {

namespace {

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
        if (it >= 0) sell_slice_learned<1>(P, it, lane, round, kind, change, tight_ctr, ws, L);
        else split_partial<1>(P, -it - 1, lane, round, kind != kRoundFull, change, tight_ctr, ws);
    }
    stats_flush(P, ws, lane);
    if (lane == 0 && L.marked) atomicAdd(marked_ctr, L.marked);
}

// Commit changed variables (and the round's row-side infeasibility, as in
// finalize_words); mark their rows for the next round: SELL rows become (or
// stay) dirty, split rows get the next round's stamp.
__device__ __forceinline__ void learned_finalize(const DevProblem &P, int round, bool push, int tid,
                                                 int nthreads) {
    unsigned long long changed = 0;
    if (tid == 0 && P.flags[0].infeasible_row != INT_MAX) P.flags[0].infeasible = 1;
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
            store_bnd32<1>(P, j, b, round);
            if (var_infeasible(b.x, b.y)) {
                P.flags[0].infeasible = 1;
                atomicMin(&P.flags[0].infeasible_var, j);
            }
            if (!push) continue;
            for (int k = __ldg(P.var_ptr + j); k < __ldg(P.var_ptr + j + 1); k++)
                learned_mark_position(P, __ldg(&P.var_ent[k].pos), round + 1);
        }
    }
    flush_changed(P, changed);
}

__global__ void __launch_bounds__(kCtaThreads, 3) k_megakernel_learned(DevProblem P) {
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
            if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
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
                if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
                if (*((volatile int *)exact)) {
                    exact_phase(P, round, q + 2, change, tight, mine, lane);
                    if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
                }
            }
            const unsigned t = *((volatile unsigned *)tight);
            const bool certified = learned_certifies(kind, t);
            const unsigned long long marked =
                    *((volatile unsigned long long *)&P.flags[1 + par].rows_deferred);
            const int next = learned_next_kind(kind, t, marked, P.n_srows, P.use_marking);
            learned_finalize(P, round, !certified && next != kRoundFull && round < P.max_rounds,
                             blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
            if (blockIdx.x == 0 && threadIdx.x == 0) P.flags[0].rounds = round;
            if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
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

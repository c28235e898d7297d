// gdp_round.cu -- one Jacobi propagation round on sm_103a, as phase kernels
// (CPU_LOOP and GPU_LOOP drivers) and as a persistent cooperative megakernel
// that runs every round in one launch (MEGAKERNEL driver). The round's device
// functions live in gdp_round.cuh.
#include <algorithm>

#include "gdp_round.cuh"

namespace gdp {

namespace {

// ---- phase kernels (CPU_LOOP / GPU_LOOP) -----------------------------------
__global__ void __launch_bounds__(kCtaThreads, 4) k_activity(DevProblem P) {
    __shared__ WarpSmem ws[kWarpsPerCta];
    const int round = P.flags[0].rounds;
    if (P.flags[0].infeasible) return;
    activity_phase(P, round, P.flags[0].mark_cur != 0, P.queue + 0, &P.flags[0].change, &P.flags[0].tight,
                   ws[threadIdx.x >> 5], threadIdx.x & 31);
}

__global__ void __launch_bounds__(kCtaThreads, 4) k_candidates(DevProblem P) {
    __shared__ WarpSmem ws[kWarpsPerCta];
    const int round = P.flags[0].rounds;
    if (P.flags[0].infeasible) return;
    // the multi-tile rows' tiles (1,024 non-zeros each) first, the deferred
    // exact rows (at most split_tile non-zeros, mostly short) after them: the
    // heavy items do not end up as the phase's tail
    candidate_phase(P, round, P.flags[0].mark_cur != 0, P.queue + 1, &P.flags[0].exact, ws[threadIdx.x >> 5],
                    threadIdx.x & 31);
    if (exact_rows_queued(P, 0))
        exact_rows_phase(P, 0, &P.flags[0].change, &P.flags[0].tight, ws[threadIdx.x >> 5], threadIdx.x & 31);
}

__global__ void __launch_bounds__(kCtaThreads, 4) k_exact(DevProblem P) {
    __shared__ WarpSmem ws[kWarpsPerCta];
    const int round = P.flags[0].rounds;
    if (P.flags[0].infeasible || P.flags[0].exact == 0) return;
    exact_phase(P, round, P.queue + 2, &P.flags[0].change, &P.flags[0].tight, ws[threadIdx.x >> 5],
                threadIdx.x & 31);
}

// Every thread derives the same next-round mode from the final tightening count.
__global__ void __launch_bounds__(256) k_finalize(DevProblem P) {
    const bool push = next_round_marked(P, P.flags[0].tight);
    finalize_words(P, P.flags[0].rounds, push, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Starts a round: counts it, takes the mode the previous finalize chose,
// clears the change flag, tightening count and work counters (unless the
// propagation is already infeasible).
__global__ void k_round_begin(DevProblem P) {
    if (P.flags[0].infeasible) return;
    const int r = P.flags[0].rounds;
    P.flags[0].mark_cur = r > 0 && next_round_marked(P, P.flags[0].tight);
    P.flags[0].change = 0;
    P.flags[0].tight = 0u;
    P.flags[0].exact = 0;
    P.flags[0].rounds = r + 1;
    P.queue[0] = 0u;
    P.queue[1] = 0u;
    P.queue[2] = 0u;
    if (P.xctr)
        for (int i = 0; i < 16; i++) P.xctr[i] = 0u;
}

// GPU_LOOP: decides whether the graph's WHILE node runs another round.
__global__ void k_condition(DevProblem P, cudaGraphConditionalHandle h) {
    const RoundFlags &f = P.flags[0];
    const bool more = f.change && !f.infeasible && f.rounds < P.max_rounds;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

__global__ void __launch_bounds__(256) k_check_bounds(DevProblem P) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < P.n; j += gridDim.x * blockDim.x) {
        const double2 b = P.bnd[j];
        if (var_infeasible(b.x, b.y)) {
            P.flags[0].infeasible = 1;
            atomicMin(&P.flags[0].infeasible_var, j);
        }
    }
}

__global__ void __launch_bounds__(256) k_interleave(DevProblem P, const double *lb, const double *ub) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < P.n; j += gridDim.x * blockDim.x) {
        const double2 b = make_double2(lb[j], ub[j]);
        P.bnd[j] = b;
        P.bnd_nxt[j] = b;
        store_bnd32<1>(P, j, b, 0);
    }
}

__global__ void __launch_bounds__(256) k_deinterleave(DevProblem P, double *lb, double *ub) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < P.n; j += gridDim.x * blockDim.x) {
        const double2 b = P.bnd[j];
        lb[j] = b.x;
        ub[j] = b.y;
    }
}

// Copies n bound pairs into the caller's arrays (host memory the device
// reaches directly).
__global__ void __launch_bounds__(256) k_copy_out(const double *lb, const double *ub, double *lb_out,
                                                  double *ub_out, int n) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        lb_out[j] = lb[j];
        ub_out[j] = ub[j];
    }
}

__global__ void __launch_bounds__(256) k_mark_all(DevProblem P) {
    const int npos = P.n_srows + P.n_lrows;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npos; p += gridDim.x * blockDim.x) P.mark[p] = 0;
    if (P.lrow_margin)  // no drift bound carried over from an earlier propagation
        for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < P.n_lrows; r += gridDim.x * blockDim.x) {
            P.lrow_margin[r] = -1.0;
            P.lrow_drift[r] = 0.0;
            P.lrow_skip[r] = 0;
        }
}

// ---- megakernel -----------------------------------------------------------
#ifdef GDP_PHASE_TIMERS
// Stamp k of round r by one thread (0: round start, 1: after phase A's
// barrier, 2: after B's, 3: after C's, 4: after F's, with the cumulative
// processed rows, non-zeros and exact non-zeros in slots 5-7).
__device__ __forceinline__ void timer_stamp(const DevProblem &P, int round, int k) {
    if (blockIdx.x != 0 || threadIdx.x != 0 || round >= kTimerRounds) return;
    unsigned long long *w = g_timer_wall + round * kTimerSlots;
    w[k] = timer_now();
    if (k == 4) {
        w[5] = *((volatile unsigned long long *)&P.flags[0].rows_proc);
        w[6] = *((volatile unsigned long long *)&P.flags[0].nnz_proc);
        w[7] = *((volatile unsigned long long *)&P.flags[0].nnz_exact);
    }
}
// adds the warp's time in phase k of round r since t0 (0: A, 1: B multi-tile
// rows, 2: B deferred exact rows, 3: C, 4: F), and keeps the longest single
// warp's time of the phase group in slot 5 (A), 6 (B) or 7 (C and F)
__device__ __forceinline__ void timer_busy(int lane, int round, int k, unsigned long long t0) {
    if (lane == 0 && round < kTimerRounds) {
        const unsigned long long dt = timer_now() - t0;
        atomicAdd(&g_timer_busy[round * kTimerSlots + k], dt);
        atomicMax(&g_timer_busy[round * kTimerSlots + (k == 0 ? 5 : k <= 2 ? 6 : 7)], dt);
    }
}
#else
__device__ __forceinline__ void timer_stamp(const DevProblem &, int, int) {}
__device__ __forceinline__ void timer_busy(int, int, int, unsigned long long) {}
#endif

// Round loop on the device. flags[0] holds the sticky state; flags[1 + (round
// & 1)] the per-round change flag, tightening and exact-row counts, and
// queue[4 * (round & 1) + phase] the per-round work counters, double-buffered
// so that nothing a CTA may still read is cleared: the next round's slots are cleared after the current
// round's first barrier, which every CTA passes only after finishing the
// previous round.
// W warps per CTA; with 24 / W resident CTAs per SM every instance holds about
// 24 warps per SM under the same register budget.
template <int W>
__global__ void __launch_bounds__(32 * W, 24 / W) k_megakernel(DevProblem P) {
    __shared__ WarpSmem ws[W];
    const int lane = threadIdx.x & 31;
    WarpSmem &mine = ws[threadIdx.x >> 5];
    int *err = &P.flags[0].error;
    int last_change = 0;
    bool marked = false;  // round 1 processes every row
    if (*((volatile int *)&P.flags[0].infeasible) == 0) {
        for (int round = 1; round <= P.max_rounds; round++) {
            const int par = round & 1;
            int *change = &P.flags[1 + par].change;
            unsigned *tight = &P.flags[1 + par].tight;
            int *exact = &P.flags[1 + par].exact;
            unsigned *q = P.queue + 4 * par;
            timer_stamp(P, round, 0);
            unsigned long long t0 = timer_now();
            activity_phase(P, round, marked, q + 0, change, tight, mine, lane, par);
            timer_busy(lane, round, 0, t0);
            if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
            timer_stamp(P, round, 1);
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                P.flags[1 + (par ^ 1)].change = 0;
                P.flags[1 + (par ^ 1)].tight = 0u;
                P.flags[1 + (par ^ 1)].exact = 0;
                P.queue[4 * (par ^ 1) + 0] = 0u;
                P.queue[4 * (par ^ 1) + 1] = 0u;
                P.queue[4 * (par ^ 1) + 2] = 0u;
                if (P.xctr)
                    for (int i = 0; i < 16; i++) P.xctr[16 * (par ^ 1) + i] = 0u;
            }
            const bool xrows = exact_rows_queued(P, par);
            if (xrows || P.n_mtiles) {
                t0 = timer_now();
                if (P.n_mtiles) candidate_phase(P, round, marked, q + 1, exact, mine, lane);  // heavy items first
                timer_busy(lane, round, 1, t0);
                t0 = timer_now();
                if (xrows) exact_rows_phase(P, par, change, tight, mine, lane);
                timer_busy(lane, round, 2, t0);
                if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
                timer_stamp(P, round, 2);
                if (P.n_mtiles && *((volatile int *)exact)) {
                    t0 = timer_now();
                    exact_phase(P, round, q + 2, change, tight, mine, lane);
                    timer_busy(lane, round, 3, t0);
                    if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
                    timer_stamp(P, round, 3);
                }
            }
            marked = next_round_marked(P, *((volatile unsigned *)tight));
            t0 = timer_now();
            finalize_words(P, round, marked, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
            timer_busy(lane, round, 4, t0);
            if (blockIdx.x == 0 && threadIdx.x == 0) P.flags[0].rounds = round;
            if (!grid_barrier(P.barrier, err, P.spin_limit)) return;
            timer_stamp(P, round, 4);
            last_change = *((volatile int *)change);
            const int infeasible = *((volatile int *)&P.flags[0].infeasible);
            if (!last_change || infeasible) break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.flags[0].change = last_change;
        P.flags[0].done = 1;
    }
}

}  // namespace

// ---- phase timers ---------------------------------------------------------

int phase_timers_clear() {
#ifdef GDP_PHASE_TIMERS
    static const unsigned long long zero[kTimerRounds * kTimerSlots] = {};
    cudaError_t e = cudaMemcpyToSymbol(g_timer_wall, zero, sizeof(zero));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_timer_busy, zero, sizeof(zero));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_timer_pass, zero, sizeof(unsigned long long) * kTimerPass);
    return (int)e;
#else
    return -1;
#endif
}

int phase_timers_read(unsigned long long *wall, unsigned long long *busy, unsigned long long *pass, int rounds) {
#ifdef GDP_PHASE_TIMERS
    const size_t k = sizeof(unsigned long long) * kTimerSlots * (size_t)std::min(std::max(rounds, 0), kTimerRounds);
    cudaError_t e = cudaSuccess;
    if (wall) e = cudaMemcpyFromSymbol(wall, g_timer_wall, k);
    if (busy && e == cudaSuccess) e = cudaMemcpyFromSymbol(busy, g_timer_busy, k);
    if (pass && e == cudaSuccess) e = cudaMemcpyFromSymbol(pass, g_timer_pass, sizeof(unsigned long long) * kTimerPass);
    return (int)e;
#else
    (void)wall, (void)busy, (void)pass, (void)rounds;
    return -1;
#endif
}

// ---- launchers ------------------------------------------------------------

int launch_check_bounds(const DevProblem &P, int blocks, cudaStream_t s) {
    if (P.n == 0) return 0;
    k_check_bounds<<<blocks, 256, 0, s>>>(P);
    return (int)cudaGetLastError();
}

int launch_interleave(const DevProblem &P, const double *lb, const double *ub, int blocks, cudaStream_t s) {
    k_interleave<<<blocks, 256, 0, s>>>(P, lb, ub);
    return (int)cudaGetLastError();
}

int launch_copy_out(const double *lb, const double *ub, double *lb_out, double *ub_out, int n, int blocks,
                    cudaStream_t s) {
    if (n > 0) k_copy_out<<<blocks, 256, 0, s>>>(lb, ub, lb_out, ub_out, n);
    return (int)cudaGetLastError();
}

int launch_deinterleave(const DevProblem &P, double *lb, double *ub, int blocks, cudaStream_t s) {
    k_deinterleave<<<blocks, 256, 0, s>>>(P, lb, ub);
    return (int)cudaGetLastError();
}

int launch_mark_all(const DevProblem &P, int blocks, cudaStream_t s) {
    if (!P.use_marking || P.n_srows + P.n_lrows == 0) return 0;
    k_mark_all<<<blocks, 256, 0, s>>>(P);
    return (int)cudaGetLastError();
}

int launch_round_begin(const DevProblem &P, cudaStream_t s) {
    k_round_begin<<<1, 1, 0, s>>>(P);
    return (int)cudaGetLastError();
}

int launch_activity_phase(const DevProblem &P, int blocks, cudaStream_t s) {
    if (P.n_items == 0) return 0;
    k_activity<<<blocks, kCtaThreads, 0, s>>>(P);
    return (int)cudaGetLastError();
}

int launch_candidate_phase(const DevProblem &P, int blocks, cudaStream_t s) {
    if (P.n_mtiles == 0 && !P.defer_exact) return 0;
    k_candidates<<<blocks, kCtaThreads, 0, s>>>(P);
    return (int)cudaGetLastError();
}

int launch_exact_phase(const DevProblem &P, int blocks, cudaStream_t s) {
    if (P.n_mtiles == 0) return 0;
    k_exact<<<blocks, kCtaThreads, 0, s>>>(P);
    return (int)cudaGetLastError();
}

int launch_finalize(const DevProblem &P, int blocks, cudaStream_t s) {
    if (P.n_chg_words == 0) return 0;
    k_finalize<<<blocks, 256, 0, s>>>(P);
    return (int)cudaGetLastError();
}

int launch_condition(const DevProblem &P, unsigned long long handle, cudaStream_t s) {
    k_condition<<<1, 1, 0, s>>>(P, (cudaGraphConditionalHandle)handle);
    return (int)cudaGetLastError();
}

namespace {
const void *megakernel_of(int cta_warps) {
    switch (cta_warps) {
        case 4: return (const void *)k_megakernel<4>;
        case 16: return (const void *)k_megakernel<16>;
        default: return (const void *)k_megakernel<8>;
    }
}
}  // namespace

int phase_occupancy(int *act, int *cand, int *mega, int cta_warps) {
    // the megakernel's shared memory (warp queues and row constants, ~3.6 KB
    // per warp, ~24 warps per SM) is small: prefer a carveout that just holds
    // it, the rest of the 256 KB per SM serving as L1 for the element streams
    const void *mk = megakernel_of(cta_warps);
    cudaError_t e = cudaFuncSetAttribute(mk, cudaFuncAttributePreferredSharedMemoryCarveout, 40);
    if (e != cudaSuccess) return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(act, k_activity, kCtaThreads, 0);
    if (e != cudaSuccess) return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(cand, k_exact, kCtaThreads, 0);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(mega, mk, 32 * cta_warps, 0);
}

int launch_megakernel(const DevProblem &P, int grid, int cta_warps, cudaStream_t s) {
    DevProblem Pc = P;
    void *args[] = {&Pc};
    return (int)cudaLaunchCooperativeKernel(megakernel_of(cta_warps), dim3(grid), dim3(32 * cta_warps), args, 0,
                                            s);
}

}  // namespace gdp

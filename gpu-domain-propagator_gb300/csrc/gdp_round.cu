// gdp_round.cu -- one Jacobi propagation round on sm_103a, as standalone
// kernels (CPU_LOOP / GPU_LOOP drivers) and as a persistent cooperative
// megakernel that runs every round in one launch (MEGAKERNEL driver).
//
// A round reads the round-start bounds (cur), writes every tightening into nxt
// with an FP64 min/max atomic and flags the variable in a bitmap; the finalize
// phase copies the flagged variables nxt -> cur and applies the
// infeasibility rule. The result is independent of scheduling: each row's sums
// are computed in a fixed order from the snapshot and min/max commute.
// Reference: the round body of GPUAtomicDomainPropagation
// (src/kernels/atomic_kernel.cuh:9-450) and of the megakernel
// (src/kernels/atomic_megakernel.cuh:14-490), re-planned for a snapshot
// (deterministic) schedule.
#include <climits>
#include <cuda_runtime.h>

#include "gdp_device.cuh"
#include "gdp_internal.h"

namespace gdp {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void mark_changed(const DevProblem &P, int j) {
    atomicOr(P.chg + (j >> 5), 1u << (j & 31));
}

__device__ __forceinline__ void to_acts(RowActs &a, const RowActsPOD &p) {
    a.minact = p.minact; a.maxact = p.maxact; a.maxactdelta = p.maxactdelta;
    a.minact_inf = p.minact_inf; a.maxact_inf = p.maxact_inf;
}

// Apply one element's candidates; returns true if it tightened something.
__device__ __forceinline__ bool apply_candidates(const DevProblem &P, const RowCand &rc, int j,
                                                 double coeff) {
    const double lb = __ldg(P.lb + j), ub = __ldg(P.ub + j);
    bool lt, ut;
    double nl, nu;
    tighten_variable(coeff, rc, __ldg(P.is_cont + j) != 0, lb, ub, lt, nl, ut, nu);
    if (lt) atomic_max_f64(P.lb_nxt + j, nl);
    if (ut) atomic_min_f64(P.ub_nxt + j, nu);
    if (lt || ut) {
        mark_changed(P, j);
        return true;
    }
    return false;
}

// ---- thread rows: one warp per slice, one lane per row ---------------------
__device__ __forceinline__ void sell_slice(const DevProblem &P, int slice, int lane, int change_slot) {
    const int r = slice * 32 + lane;
    const bool valid = r < P.n_srows;
    const int len = valid ? __ldg(P.srow_len + r) : 0;
    const long long base = __ldg(P.slice_ptr + slice) + lane;
    const int *__restrict__ col = P.sell_col + base;
    const double *__restrict__ val = P.sell_val + base;

    RowActs a;
    acts_init(a);
#pragma unroll 4
    for (int k = 0; k < len; k++) {
        const int j = __ldg(col + 32 * (long long)k);
        const double c = __ldg(val + 32 * (long long)k);
        acts_add(a, c, __ldg(P.lb + j), __ldg(P.ub + j));
    }
    bool tight = false;
    if (valid) {
        const double lhs = __ldg(P.srow_lhs + r), rhs = __ldg(P.srow_rhs + r);
        if (can_cons_be_tightened(a, lhs, rhs)) {
            const RowCand rc = row_cand(a, lhs, rhs);
            for (int k = 0; k < len; k++)
                tight |= apply_candidates(P, rc, __ldg(col + 32 * (long long)k), __ldg(val + 32 * (long long)k));
        }
    }
    if (__any_sync(kFull, tight) && lane == 0) P.flags[change_slot].change = 1;
}

// ---- split rows: one CTA per tile -----------------------------------------
__device__ __forceinline__ void combine(RowActs &a, const RowActs &b) {
    a.minact = dadd(a.minact, b.minact);
    a.maxact = dadd(a.maxact, b.maxact);
    a.maxactdelta = fmax(a.maxactdelta, b.maxactdelta);
    a.minact_inf += b.minact_inf;
    a.maxact_inf += b.maxact_inf;
}

__device__ __forceinline__ RowActs shfl_down(const RowActs &a, int off) {
    RowActs b;
    b.minact = __shfl_down_sync(kFull, a.minact, off);
    b.maxact = __shfl_down_sync(kFull, a.maxact, off);
    b.maxactdelta = __shfl_down_sync(kFull, a.maxactdelta, off);
    b.minact_inf = __shfl_down_sync(kFull, a.minact_inf, off);
    b.maxact_inf = __shfl_down_sync(kFull, a.maxact_inf, off);
    return b;
}

// Partial activities of tile t. Thread i sums elements i, i+256, ... in order;
// the warp tree and the warp-order combine are fixed, so the partial is
// deterministic. Split rows keep the exact max of |a|(ub-lb) (a sequential
// EPS-max is not defined for a tree).
__device__ void split_partial(const DevProblem &P, int t, RowActsPOD *smem) {
    const int b = __ldg(P.tile_begin + t), e = __ldg(P.tile_end + t);
    RowActs a;
    acts_init(a);
    for (int k = b + (int)threadIdx.x; k < e; k += kSplitThreads) {
        const int j = __ldg(P.lcol + k);
        const double c = __ldg(P.lval + k);
        const double lb = __ldg(P.lb + j), ub = __ldg(P.ub + j);
        const double delta = dmul(fabs(c), dsub(ub, lb));
        a.maxactdelta = fmax(a.maxactdelta, delta);
        const bool pos = c > kEps;
        const bool min_inf = pos ? is_neginf(lb) : is_posinf(ub);
        const bool max_inf = pos ? is_posinf(ub) : is_neginf(lb);
        a.minact_inf += min_inf;
        a.maxact_inf += max_inf;
        const bool gt0 = c > 0.0;
        if (!min_inf) a.minact = dadd(a.minact, dmul(c, gt0 ? lb : ub));
        if (!max_inf) a.maxact = dadd(a.maxact, dmul(c, gt0 ? ub : lb));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) combine(a, shfl_down(a, off));
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        smem[warp].minact = a.minact; smem[warp].maxact = a.maxact;
        smem[warp].maxactdelta = a.maxactdelta;
        smem[warp].minact_inf = a.minact_inf; smem[warp].maxact_inf = a.maxact_inf;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        RowActs s;
        to_acts(s, smem[0]);
        for (int w = 1; w < kSplitThreads / 32; w++) {
            RowActs o;
            to_acts(o, smem[w]);
            combine(s, o);
        }
        RowActsPOD out;
        out.minact = s.minact; out.maxact = s.maxact; out.maxactdelta = s.maxactdelta;
        out.minact_inf = s.minact_inf; out.maxact_inf = s.maxact_inf;
        P.tile_part[t] = out;
    }
    __syncthreads();
}

// Candidates of tile t from its row's combined activities (tiles combined in
// tile order by every thread: identical values, no extra barrier).
__device__ void split_cand(const DevProblem &P, int t, int change_slot) {
    const int r = __ldg(P.tile_row + t);
    const int t0 = __ldg(P.lrow_tile0 + r), t1 = __ldg(P.lrow_tile0 + r + 1);
    RowActs a;
    to_acts(a, P.tile_part[t0]);
    for (int u = t0 + 1; u < t1; u++) {
        RowActs o;
        to_acts(o, P.tile_part[u]);
        combine(a, o);
    }
    const double lhs = __ldg(P.lrow_lhs + r), rhs = __ldg(P.lrow_rhs + r);
    if (!can_cons_be_tightened(a, lhs, rhs)) return;
    const RowCand rc = row_cand(a, lhs, rhs);
    const int b = __ldg(P.tile_begin + t), e = __ldg(P.tile_end + t);
    bool tight = false;
    for (int k = b + (int)threadIdx.x; k < e; k += blockDim.x)
        tight |= apply_candidates(P, rc, __ldg(P.lcol + k), __ldg(P.lval + k));
    if (__any_sync(kFull, tight) && (threadIdx.x & 31) == 0) P.flags[change_slot].change = 1;
}

// Copy changed variables nxt -> cur, apply the infeasibility rule, clear the
// bitmap. Grid-stride over bitmap words.
__device__ void finalize_words(const DevProblem &P, int tid, int nthreads) {
    int changed = 0;
    for (int w = tid; w < P.n_chg_words; w += nthreads) {
        unsigned bits = P.chg[w];
        if (!bits) continue;
        P.chg[w] = 0u;
        changed += __popc(bits);
        while (bits) {
            const int bit = __ffs(bits) - 1;
            bits &= bits - 1;
            const int j = w * 32 + bit;
            const double l = P.lb_nxt[j], u = P.ub_nxt[j];
            P.lb[j] = l;
            P.ub[j] = u;
            if (var_infeasible(l, u)) {
                P.flags[0].infeasible = 1;
                atomicMin(&P.flags[0].infeasible_var, j);
            }
        }
    }
    if (changed) atomicAdd(&P.flags[0].changed_vars, changed);
}

// ---- standalone kernels ---------------------------------------------------
__global__ void __launch_bounds__(32 * kSellWarpsPerCta) k_sell_round(DevProblem P) {
    const int slice = blockIdx.x * kSellWarpsPerCta + (threadIdx.x >> 5);
    if (slice >= P.n_slices) return;
    sell_slice(P, slice, threadIdx.x & 31, 0);
}

__global__ void __launch_bounds__(kSplitThreads) k_split_partial(DevProblem P) {
    __shared__ RowActsPOD smem[kSplitThreads / 32];
    split_partial(P, blockIdx.x, smem);
}

__global__ void __launch_bounds__(kSplitThreads) k_split_cand(DevProblem P) {
    split_cand(P, blockIdx.x, 0);
}

__global__ void __launch_bounds__(kFinalizeThreads) k_finalize(DevProblem P) {
    finalize_words(P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Zero the round's change flag and count the round.
__global__ void k_round_begin(DevProblem P) {
    P.flags[0].change = 0;
    P.flags[0].rounds += 1;
}

// ---- megakernel -----------------------------------------------------------
// Grid barrier with a bounded wait: thread 0 of each CTA reads the barrier
// generation, arrives, and spins until the generation moves. Any CTA that
// waits longer than kSpinLimitCycles (or sees another CTA's error) records
// kErrBarrierTimeout and every CTA leaves the round loop at its next barrier.
constexpr long long kSpinLimitCycles = 4000000000LL;  // about 2 s at 2 GHz

__device__ bool grid_barrier(unsigned *bar, int *error) {
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
                if (clock64() - t0 > kSpinLimitCycles) {
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

// Round loop on the device. flags[0] holds the sticky state (rounds,
// infeasibility, error, last change); flags[1 + (round & 1)].change is the
// per-round change flag, double-buffered so that no CTA can clear a flag
// another CTA has not read yet (the slot of round r+1 is cleared after round
// r's first barrier, which every CTA passes only after reading round r-1's).
__global__ void __launch_bounds__(kMegaThreads) k_megakernel(DevProblem P) {
    __shared__ RowActsPOD smem[kMegaThreads / 32];
    const int n_groups = (P.n_slices + kSellWarpsPerCta - 1) / kSellWarpsPerCta;
    const int n_items = P.n_tiles + n_groups;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *err = &P.flags[0].error;
    int last_change = 0;
    if (*((volatile int *)&P.flags[0].infeasible) == 0) {
        for (int round = 1; round <= P.max_rounds; round++) {
            const int slot = 1 + (round & 1);
            // phase A: split-row partials, then thread-row slices
            for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
                if (item < P.n_tiles) {
                    split_partial(P, item, smem);
                } else {
                    const int slice = (item - P.n_tiles) * kSellWarpsPerCta + warp;
                    if (slice < P.n_slices) sell_slice(P, slice, lane, slot);
                }
            }
            if (!grid_barrier(P.barrier, err)) return;
            if (blockIdx.x == 0 && threadIdx.x == 0) P.flags[1 + ((round + 1) & 1)].change = 0;
            // phase B: split-row candidates
            for (int t = blockIdx.x; t < P.n_tiles; t += gridDim.x) split_cand(P, t, slot);
            if (!grid_barrier(P.barrier, err)) return;
            // phase C: commit changed variables, infeasibility rule
            finalize_words(P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
            if (blockIdx.x == 0 && threadIdx.x == 0) P.flags[0].rounds = round;
            if (!grid_barrier(P.barrier, err)) return;
            last_change = *((volatile int *)&P.flags[slot].change);
            const int infeasible = *((volatile int *)&P.flags[0].infeasible);
            if (!last_change || infeasible) break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.flags[0].change = last_change;
        P.flags[0].done = 1;
    }
}

// Initial infeasibility check over every variable (before round 1).
__global__ void __launch_bounds__(kFinalizeThreads) k_check_bounds(DevProblem P) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < P.n; j += gridDim.x * blockDim.x) {
        if (var_infeasible(P.lb[j], P.ub[j])) {
            P.flags[0].infeasible = 1;
            atomicMin(&P.flags[0].infeasible_var, j);
        }
    }
}

}  // namespace

// ---- launchers ------------------------------------------------------------
int launch_round_begin(const DevProblem &P, void *stream) {
    k_round_begin<<<1, 1, 0, (cudaStream_t)stream>>>(P);
    return (int)cudaGetLastError();
}

int launch_check_bounds(const DevProblem &P, int blocks, void *stream) {
    if (P.n == 0) return 0;
    k_check_bounds<<<blocks, kFinalizeThreads, 0, (cudaStream_t)stream>>>(P);
    return (int)cudaGetLastError();
}

int launch_sell_round(const DevProblem &P, void *stream) {
    if (P.n_slices == 0) return 0;
    const int grid = (P.n_slices + kSellWarpsPerCta - 1) / kSellWarpsPerCta;
    k_sell_round<<<grid, 32 * kSellWarpsPerCta, 0, (cudaStream_t)stream>>>(P);
    return (int)cudaGetLastError();
}

int launch_split_partial(const DevProblem &P, void *stream) {
    if (P.n_tiles == 0) return 0;
    k_split_partial<<<P.n_tiles, kSplitThreads, 0, (cudaStream_t)stream>>>(P);
    return (int)cudaGetLastError();
}

int launch_split_cand(const DevProblem &P, void *stream) {
    if (P.n_tiles == 0) return 0;
    k_split_cand<<<P.n_tiles, kSplitThreads, 0, (cudaStream_t)stream>>>(P);
    return (int)cudaGetLastError();
}

int launch_finalize(const DevProblem &P, int finalize_blocks, void *stream) {
    if (P.n_chg_words == 0) return 0;
    k_finalize<<<finalize_blocks, kFinalizeThreads, 0, (cudaStream_t)stream>>>(P);
    return (int)cudaGetLastError();
}

int megakernel_occupancy(int block, int *blocks_per_sm) {
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_megakernel, block, 0);
}

int launch_megakernel(const DevProblem &P, int grid, int block, void *stream) {
    DevProblem Pc = P;
    void *args[] = {&Pc};
    return (int)cudaLaunchCooperativeKernel((const void *)k_megakernel, dim3(grid), dim3(block), args, 0,
                                            (cudaStream_t)stream);
}

}  // namespace gdp

// gdp_batch.cu -- the batched engine: many problems (instances) or many
// bound vectors of one problem (branch-and-bound nodes) propagated together
// in one persistent cooperative launch.
//
// Each batch member ("unit") is a DevProblem: its own bounds, change bitmap,
// marks and round flags, over its own layout (instances) or a layout shared
// with the other units (nodes). Every unit follows exactly the Jacobi rounds
// it would follow alone -- units never read each other's bounds -- so its
// bounds, round count and infeasibility verdict equal those of a
// single-problem propagation. What the batch adds is scheduling:
//   * one work list per round across all units: (unit, slice/tile) entries
//     queued when a changed variable marks a row, plus full sweeps (a
//     virtual range over a unit's work items) for units whose last round
//     tightened many bounds;
//   * a unit leaves the loop the round it converges or turns infeasible, so
//     short and long propagations share the launch without waiting rounds;
//   * nodes start from the marks of the variables whose bounds differ from a
//     certified fixpoint of the same problem (every other row is at its
//     fixpoint already and would find nothing).
// The round loop runs in one cooperative kernel (grid barriers between the
// phases, bounded waits) and the whole device part of a call is captured once
// into a CUDA graph and replayed.
//
// Reference: the reference propagates one problem per call
// (include/interface.h:10-251); its GPU round loop is
// src/propagators/GPU_propagator.cuh:160-255.
#include "gdp_batch.h"

#include <algorithm>
#include <chrono>
#include <cstring>

#include "gdp_learned.cuh"

namespace gdp {

namespace {

// Finds the unit whose half-open range [base[u], base[u+1]) holds x.
__device__ __forceinline__ int find_unit(const int *base, int n_units, int x) {
    int lo = 0, hi = n_units;  // base[lo] <= x < base[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(base + mid) <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void push_entry(const BatchDev &B, int par, int u, int item) {
    const unsigned idx = atomicAdd(B.tail + par, 1u);
    if (idx >= B.cap_entries) {
        atomicExch(B.error, (int)kErrQueueOverflow);
        return;
    }
    B.entries[(size_t)par * B.cap_entries + idx] = ((unsigned long long)(unsigned)u << 32) | (unsigned)item;
}

__device__ __forceinline__ void push_tile(unsigned long long *q, unsigned *tail, unsigned cap, int *error, int u,
                                          int t) {
    const unsigned idx = atomicAdd(tail, 1u);
    if (idx >= cap) {
        atomicExch(error, (int)kErrQueueOverflow);
        return;
    }
    q[idx] = ((unsigned long long)(unsigned)u << 32) | (unsigned)t;
}

// Queues row position p of unit u for round `stamp` (its mark is already set):
// the slice holding it once per round, or every tile of a split row.
__device__ __forceinline__ void queue_position(const BatchDev &B, const DevProblem &Pu, int u, int p, int stamp) {
    const int par = stamp & 1;
    if (p < Pu.n_srows) {
        const int s = __ldg(Pu.pos_slice + p);
        if (atomicExch(Pu.slice_stamp + s, stamp) != stamp) push_entry(B, par, u, s);
    } else {
        const int row = p - Pu.n_srows;
        for (int t = __ldg(Pu.lrow_tile0 + row); t < __ldg(Pu.lrow_tile0 + row + 1); t++) push_entry(B, par, u, -t - 1);
    }
}

// Learned units: variable j of unit u changed; its SELL rows turn dirty and
// their slices are queued for round `stamp`, its split rows are marked and
// their tiles queued (as in learned_mark_position).
__device__ __forceinline__ void mark_var_rows_learned(const BatchDev &B, const DevProblem &Pu, int u, int j,
                                                      int stamp) {
    for (int k = __ldg(Pu.var_ptr + j); k < __ldg(Pu.var_ptr + j + 1); k++) {
        const int p = __ldg(&Pu.var_ent[k].pos);
        if (p < Pu.n_srows) {
            atomicAdd(Pu.dcount + p, 1);
            if (Pu.dirty[p] == 0) atomicCAS(Pu.dirty + p, 0, stamp);
            const int s = __ldg(Pu.pos_slice + p);
            if (atomicExch(Pu.slice_stamp + s, stamp) != stamp) push_entry(B, stamp & 1, u, s);
        } else if (atomicExch(Pu.mark + p, stamp) != stamp) {
            queue_position(B, Pu, u, p, stamp);
        }
    }
}

// Marks the rows of variable j of unit u for round `stamp` and queues them.
__device__ __forceinline__ void mark_var_rows(const BatchDev &B, const DevProblem &Pu, int u, int j, int stamp) {
    for (int k = __ldg(Pu.var_ptr + j); k < __ldg(Pu.var_ptr + j + 1); k++) {
        const int p = __ldg(&Pu.var_ent[k].pos);
        if (atomicExch(Pu.mark + p, stamp) != stamp) queue_position(B, Pu, u, p, stamp);
    }
}

// One block builds the list of units swept in full in the next round, in
// unit order, with the prefix of their work-item counts.
template <class Pred>
__device__ void build_full_sweep_list(const BatchDev &B, Pred &&pred) {
    __shared__ int s_cnt[kCtaThreads / 32], s_items[kCtaThreads / 32];
    __shared__ int s_base_u, s_base_i;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) { s_base_u = 0; s_base_i = 0; }
    __syncthreads();
    for (int u0 = 0; u0 < B.n_units; u0 += kCtaThreads) {
        const int u = u0 + tid;
        const int f = (u < B.n_units && pred(u)) ? 1 : 0;
        const int items = f ? B.units[u].n_items : 0;
        int cf = f, ci = items;  // inclusive warp scans
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int a = __shfl_up_sync(kFull, cf, off), b = __shfl_up_sync(kFull, ci, off);
            if (lane >= off) { cf += a; ci += b; }
        }
        if (lane == 31) { s_cnt[wid] = cf; s_items[wid] = ci; }
        __syncthreads();
        int wf = 0, wi = 0, tf = 0, ti = 0;
        for (int w = 0; w < kCtaThreads / 32; w++) {
            if (w < wid) { wf += s_cnt[w]; wi += s_items[w]; }
            tf += s_cnt[w];
            ti += s_items[w];
        }
        if (f) {
            const int k = s_base_u + wf + cf - 1;
            B.fs_unit[k] = u;
            B.fs_prefix[k] = s_base_i + wi + ci - items;
        }
        __syncthreads();
        if (tid == 0) { s_base_u += tf; s_base_i += ti; }
        __syncthreads();
    }
    if (tid == 0) {
        B.fs_prefix[s_base_u] = s_base_i;
        B.n_fs[0] = s_base_u;
    }
}

// The kind of round r + 1 of learned unit Pu after round r.
__device__ __forceinline__ int unit_next_kind(const DevProblem &Pu, int r) {
    const RoundFlags &fr = Pu.flags[1 + (r & 1)];
    return learned_next_kind(fr.kind, fr.tight, fr.rows_deferred, Pu.n_srows, Pu.use_marking);
}
// A learned unit is finished after round r when it turned infeasible or a
// FULL or FLUSH round changed nothing (its certification).
__device__ __forceinline__ bool unit_certified(const DevProblem &Pu, int r) {
    const RoundFlags &fr = Pu.flags[1 + (r & 1)];
    return learned_certifies(fr.kind, fr.tight);
}

// Round bookkeeping of unit u after round r (every phase of r is complete).
__device__ __forceinline__ void close_round(const BatchDev &B, int u, int r) {
    RoundFlags &f0 = B.units[u].flags[0];
    if (f0.done) return;
    f0.rounds = r;
    if (B.units[u].learned == 1) {
        const bool cert = unit_certified(B.units[u], r);
        if (B.units[u].flags[1 + (r & 1)].kind == kRoundFull) f0.full_rounds += 1;
        if (f0.infeasible || cert || r >= B.max_rounds) {
            f0.done = 1;
            f0.change = (f0.infeasible || cert) ? B.units[u].flags[1 + (r & 1)].change : 1;
        }
        return;
    }
    const int ch = B.units[u].flags[1 + (r & 1)].change;
    if (f0.infeasible) {
        f0.done = 1;
        f0.change = ch;
    } else if (!ch || r >= B.max_rounds) {
        f0.done = 1;
        f0.change = ch;
    }
}

__device__ __forceinline__ bool unit_next_marked(const DevProblem &Pu, int r) {
    return next_round_marked(Pu, Pu.flags[1 + (r & 1)].tight);
}

}  // namespace

namespace {

// ---- the persistent round loop ----------------------------------------------
// Round r (par = r & 1):
//   A  work list of round r: full-sweep items (virtual range over fs_unit),
//      then queued entries[par]; split tiles of multi-tile rows go to cq.
//   B  cq: row screens of multi-tile rows; tiles needing the exact pass go to xq.
//   C  xq (only if not empty): exact partials combined, candidates.
//   F  commit changed variables of every unit; mark and queue rows for r + 1
//      (units staying on marked rounds), full-sweep list for r + 1.
// After F every CTA reads the same next-round work size and leaves together.
// kLearned: units with a model (learned == 1) run learned rounds (gdp_learned.cu)
// -- each unit its own sequence of FULL / LEARNED / FLUSH rounds, the kind of
// round r in flags[1 + (r & 1)].kind; a slice whose marked rows the model
// deferred is queued again for the next round, and a unit ends only with a FULL
// round that changes nothing, exactly as in its single-problem learned run.
// Both instantiations run 5 CTAs per SM (48 registers, spills served by L1):
// the round work is latency-bound, and on 128 chain instances the learned
// loop took 2,093 / 912 / 866 / 844 / 1,269 ms at 2 / 3 / 4 / 5 / 6 CTAs per
// SM, the plain one 590 / 567 / 561 / 566 ms at 3 / 4 / 5 / 6.
template <bool kLearned>
__global__ void __launch_bounds__(kCtaThreads, 5) k_batch_loop(BatchDev B) {
    __shared__ WarpSmem ws[kWarpsPerCta];
    __shared__ LearnSmem ls[kLearned ? kWarpsPerCta : 1];
    const int lane = threadIdx.x & 31;
    WarpSmem &mine = ws[threadIdx.x >> 5];
    LearnSmem &L = ls[kLearned ? (threadIdx.x >> 5) : 0];
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gthreads = gridDim.x * blockDim.x;
    int last = 0;
    for (int r = 1; r <= B.max_rounds; r++) {
        const int par = r & 1;
        unsigned *ctr = B.ctr + 4 * par;
        // close round r - 1 for every unit (its flags are final); the entry
        // queue of round r - 1 (parity par ^ 1) was emptied in its phase B and
        // fills for round r + 1 (phase A: slices with deferred rows, phase F)
        if (r > 1)
            for (int u = gtid; u < B.n_units; u += gthreads) close_round(B, u, r - 1);
        // ---- A
        {
            const int nfs = *((volatile int *)B.n_fs);
            const int fs_items = *((volatile int *)(B.fs_prefix + nfs));
            const int n_entries = (int)min(*((volatile unsigned *)(B.tail + par)), B.cap_entries);
            const unsigned long long *ent = B.entries + (size_t)par * B.cap_entries;
            stats_zero(mine, lane);
            for (;;) {
                const int i = warp_next(ctr + 0, lane);
                if (i >= fs_items + n_entries) break;
                int u, it;
                bool marked;
                if (i < fs_items) {
                    const int k = find_unit(B.fs_prefix, nfs, i);
                    u = B.fs_unit[k];
                    it = __ldg(B.units[u].items + (i - B.fs_prefix[k]));
                    marked = false;
                } else {
                    const unsigned long long e = ent[i - fs_items];
                    u = (int)(e >> 32);
                    it = (int)(unsigned)e;
                    marked = true;
                }
                const DevProblem &Pu = B.units[u];
                if (*((volatile int *)&Pu.flags[0].infeasible)) continue;
                int *change = &Pu.flags[1 + par].change;
                unsigned *tight = &Pu.flags[1 + par].tight;
                if (kLearned && Pu.learned == 1) {
                    const int kind = Pu.flags[1 + par].kind;
                    if (it >= 0) {
                        if (lane == 0) L.marked = 0;
                        __syncwarp();
                        const bool deferred = sell_slice_learned<0>(Pu, it, lane, r, kind, change, tight, mine, L);
                        if (lane == 0) {
                            if (L.marked) atomicAdd(&Pu.flags[1 + par].rows_deferred, L.marked);
                            if (deferred && r < B.max_rounds && atomicExch(Pu.slice_stamp + it, r + 1) != r + 1)
                                push_entry(B, par ^ 1, u, it);
                        }
                    } else if (split_partial<0>(Pu, -it - 1, lane, r, kind != kRoundFull, change, tight, mine) &&
                               lane == 0) {
                        push_tile(B.cq, B.tail + 2, B.cap_tiles, B.error, u, -it - 1);
                    }
                } else if (it >= 0) {
                    sell_slice<0>(Pu, it, lane, r, marked, change, tight, mine);
                } else if (split_partial<0>(Pu, -it - 1, lane, r, marked, change, tight, mine) && lane == 0) {
                    push_tile(B.cq, B.tail + 2, B.cap_tiles, B.error, u, -it - 1);
                }
                stats_flush(Pu, mine, lane);  // statistics belong to the item's unit
            }
        }
        if (!grid_barrier(B.barrier, B.error, B.spin_limit)) return;
        // ---- B (plus the resets for round r + 1: its slots were last used in r - 1)
        if (gtid == 0) {
            unsigned *nctr = B.ctr + 4 * (par ^ 1);
            nctr[0] = 0u; nctr[1] = 0u; nctr[2] = 0u;
            B.tail[par] = 0u;  // round r's entry queue is consumed; it fills again in round r + 1
        }
        for (int u = gtid; u < B.n_units; u += gthreads) {
            RoundFlags &fn = B.units[u].flags[1 + (par ^ 1)];
            fn.change = 0; fn.tight = 0u; fn.exact = 0;
            fn.rows_deferred = 0ULL;  // learned units: marked rows met in the round
        }
        const int n_cq = (int)min(*((volatile unsigned *)(B.tail + 2)), B.cap_tiles);
        if (n_cq) {
            for (;;) {
                const int i = warp_next(ctr + 1, lane);
                if (i >= n_cq) break;
                const unsigned long long e = B.cq[i];
                const int u = (int)(e >> 32), t = (int)(unsigned)e;
                const DevProblem &Pu = B.units[u];
                if (split_cand<0>(Pu, t, lane, r, false, &Pu.flags[1 + par].exact, mine) && lane == 0)
                    push_tile(B.xq, B.tail + 3, B.cap_tiles, B.error, u, t);
                stats_flush(Pu, mine, lane);
            }
            if (!grid_barrier(B.barrier, B.error, B.spin_limit)) return;
            // ---- C
            const int n_xq = (int)min(*((volatile unsigned *)(B.tail + 3)), B.cap_tiles);
            if (n_xq) {
                for (;;) {
                    const int i = warp_next(ctr + 2, lane);
                    if (i >= n_xq) break;
                    const unsigned long long e = B.xq[i];
                    const int u = (int)(e >> 32), t = (int)(unsigned)e;
                    const DevProblem &Pu = B.units[u];
                    split_exact<0>(Pu, t, lane, r, &Pu.flags[1 + par].change, &Pu.flags[1 + par].tight, mine);
                    stats_flush(Pu, mine, lane);
                }
                if (!grid_barrier(B.barrier, B.error, B.spin_limit)) return;
            }
        }
        // ---- F (a row recorded infeasible in round r turns into the unit's
        // verdict here, where the variable rule sets it)
        for (int u = gtid; u < B.n_units; u += gthreads)
            if (B.units[u].flags[0].infeasible_row != INT_MAX) B.units[u].flags[0].infeasible = 1;
        const bool more = r < B.max_rounds;
        if (blockIdx.x == 0) {
            if (more)
                build_full_sweep_list(B, [&](int u) {
                    const DevProblem &Pu = B.units[u];
                    if (kLearned && Pu.learned == 1)
                        return !Pu.flags[0].done && !Pu.flags[0].infeasible && !unit_certified(Pu, r) &&
                               unit_next_kind(Pu, r) == kRoundFull;
                    return !Pu.flags[0].done && Pu.flags[1 + par].change && !unit_next_marked(Pu, r);
                });
            else if (threadIdx.x == 0) {
                B.n_fs[0] = 0;
                B.fs_prefix[0] = 0;
            }
            if (threadIdx.x == 0) { B.tail[2] = 0u; B.tail[3] = 0u; }
            if (kLearned) {  // learned units that need round r + 1 even without queued work
                __shared__ int s_pend;
                if (threadIdx.x == 0) s_pend = 0;
                __syncthreads();
                for (int u = threadIdx.x; u < B.n_units; u += blockDim.x) {
                    const DevProblem &Pu = B.units[u];
                    if (Pu.learned == 1 && more && !Pu.flags[0].done && !Pu.flags[0].infeasible &&
                        !unit_certified(Pu, r))
                        atomicAdd(&s_pend, 1);
                }
                __syncthreads();
                if (threadIdx.x == 0) B.n_pending[0] = s_pend;
            }
        }
        if (kLearned)
            for (int u = gtid; u < B.n_units; u += gthreads)
                if (B.units[u].learned == 1) B.units[u].flags[1 + (par ^ 1)].kind = unit_next_kind(B.units[u], r);
        for (int w = gtid; w < B.total_words; w += gthreads) {
            const int u = find_unit(B.wbase, B.n_units, w);
            const DevProblem &Pu = B.units[u];
            const int wl = w - __ldg(B.wbase + u);
            unsigned bits = Pu.chg[wl];
            if (!bits) continue;
            Pu.chg[wl] = 0u;
            atomicAdd(&Pu.flags[0].changed_vars, (unsigned long long)__popc(bits));  // per word, per unit
            const bool lrn = kLearned && Pu.learned == 1;
            const bool push = more && (lrn ? (!unit_certified(Pu, r) && unit_next_kind(Pu, r) != kRoundFull)
                                           : unit_next_marked(Pu, r));
            while (bits) {
                const int j = wl * 32 + __ffs(bits) - 1;
                bits &= bits - 1;
                const double2 b = Pu.bnd_nxt[j];
                Pu.bnd[j] = b;
                store_bnd32<0>(Pu, j, b, r);
                if (var_infeasible(b.x, b.y)) {
                    Pu.flags[0].infeasible = 1;
                    atomicMin(&Pu.flags[0].infeasible_var, j);
                }
                if (push) {
                    if (lrn) mark_var_rows_learned(B, Pu, u, j, r + 1);
                    else mark_var_rows(B, Pu, u, j, r + 1);
                }
            }
        }
        if (!grid_barrier(B.barrier, B.error, B.spin_limit)) return;
        last = r;
        const int nfs = *((volatile int *)B.n_fs);
        const int next = *((volatile int *)(B.fs_prefix + nfs)) +
                         (int)min(*((volatile unsigned *)(B.tail + (par ^ 1))), B.cap_entries);
        const int pending = kLearned ? *((volatile int *)B.n_pending) : 0;
        if (!more || (next == 0 && pending == 0)) break;
    }
    for (int u = gtid; u < B.n_units; u += gthreads) close_round(B, u, last);
    if (gtid == 0) B.rounds_out[0] = last;
}

// Initial state of every unit: interleaved bounds, cleared bitmaps and marks,
// the round-0 infeasibility check.
__global__ void __launch_bounds__(256) k_batch_init(BatchDev B, const double *lb, const double *ub,
                                                     const long long *var_base) {
    const int u = blockIdx.y;
    const DevProblem &Pu = B.units[u];
    const long long vb = var_base[u];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < Pu.n; j += gridDim.x * blockDim.x) {
        const double2 b = make_double2(lb[vb + j], ub[vb + j]);
        Pu.bnd[j] = b;
        Pu.bnd_nxt[j] = b;
        store_bnd32<0>(Pu, j, b, 0);
        if (var_infeasible(b.x, b.y)) {
            Pu.flags[0].infeasible = 1;
            atomicMin(&Pu.flags[0].infeasible_var, j);
        }
    }
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < Pu.n_chg_words; w += gridDim.x * blockDim.x)
        Pu.chg[w] = 0u;
    const int npos = Pu.n_srows + Pu.n_lrows;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npos; p += gridDim.x * blockDim.x) Pu.mark[p] = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < Pu.n_slices; s += gridDim.x * blockDim.x)
        Pu.slice_stamp[s] = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < Pu.n_lrows; r += gridDim.x * blockDim.x)
        Pu.row_exact[r] = 0;
    if (Pu.learned == 1)
        for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < Pu.n_srows; p += gridDim.x * blockDim.x) {
            Pu.dirty[p] = 0;
            Pu.dcount[p] = 0;
            Pu.last_proc[p] = 0;
            Pu.last_tight[p] = 0;
            Pu.rstat[p] = make_float2(0.f, 0.f);
            Pu.rinfo[p] = 0u;
        }
}

// Round-1 marks of units started from a certified fixpoint `ref` of their
// problem: the rows of every variable whose bounds differ from it.
__global__ void __launch_bounds__(256) k_batch_seed_marks(BatchDev B, const double2 *ref, const int *seed_mode) {
    const int u = blockIdx.y;
    const DevProblem &Pu = B.units[u];
    if (seed_mode[u] != 1 || Pu.flags[0].infeasible) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < Pu.n; j += gridDim.x * blockDim.x) {
        const double2 a = Pu.bnd[j], b = ref[j];
        if (dbits(a.x) != dbits(b.x) || dbits(a.y) != dbits(b.y)) mark_var_rows(B, Pu, u, j, 1);
    }
}

// Round-1 full-sweep list (units with seed_mode 0) and round-0 bookkeeping.
__global__ void __launch_bounds__(kCtaThreads) k_batch_plan(BatchDev B, const int *seed_mode) {
    for (int u = threadIdx.x; u < B.n_units; u += blockDim.x) {
        RoundFlags &f0 = B.units[u].flags[0];
        if (f0.infeasible) {  // infeasible before any round
            f0.done = 1;
            f0.rounds = 0;
        }
    }
    __syncthreads();
    build_full_sweep_list(B, [&](int u) { return seed_mode[u] == 0 && !B.units[u].flags[0].infeasible; });
}

__global__ void __launch_bounds__(256) k_batch_fini(BatchDev B, double *lb, double *ub, const long long *var_base) {
    const int u = blockIdx.y;
    const DevProblem &Pu = B.units[u];
    const long long vb = var_base[u];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < Pu.n; j += gridDim.x * blockDim.x) {
        const double2 b = Pu.bnd[j];
        lb[vb + j] = b.x;
        ub[vb + j] = b.y;
    }
}

}  // namespace

// ---- launchers --------------------------------------------------------------
int batch_occupancy(int *blocks_per_sm, bool learned) {
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            blocks_per_sm, learned ? k_batch_loop<true> : k_batch_loop<false>, kCtaThreads, 0);
}

int launch_batch(const BatchDev &B, int grid, const double *lb, const double *ub, double *lb_out,
                 double *ub_out, const long long *var_base, int max_unit_n, const double2 *ref,
                 const int *seed_mode, bool learned, cudaStream_t s) {
    const dim3 vgrid((unsigned)std::max(1, std::min((max_unit_n + 255) / 256, 64)), (unsigned)B.n_units);
    k_batch_init<<<vgrid, 256, 0, s>>>(B, lb, ub, var_base);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    if (ref) {
        k_batch_seed_marks<<<vgrid, 256, 0, s>>>(B, ref, seed_mode);
        if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
    }
    k_batch_plan<<<1, kCtaThreads, 0, s>>>(B, seed_mode);
    if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
    BatchDev Bc = B;
    void *args[] = {&Bc};
    e = cudaLaunchCooperativeKernel(learned ? (const void *)k_batch_loop<true> : (const void *)k_batch_loop<false>,
                                    dim3(grid), dim3(kCtaThreads), args, 0, s);
    if (e != cudaSuccess) return (int)e;
    k_batch_fini<<<vgrid, 256, 0, s>>>(B, lb_out, ub_out, var_base);
    return (int)cudaGetLastError();
}

}  // namespace gdp

// gdp_internal.h -- device data layout shared by the host driver and kernels.
//
// HBM layout of one problem (built once per context, resident across rounds):
//  * SELL-g slices (rows up to split_tile non-zeros): rows sorted by lanes per
//    row g and length; a slice holds 32/g rows with g lanes each and stores
//    its elements column-major (step i of lane l at slice_ptr[s] + 32*i + l),
//    so a warp streams a slice with coalesced 128 B (col) / 256 B (val) loads.
//    Rows up to thread_row_max have g = 1: one lane sums the row left to
//    right -- the reference's summation order. Longer rows get g = 2..32 lanes
//    (about 32 elements per lane) and a shuffle-tree combine.
//  * split rows (len > split_tile): CSR-contiguous, cut into warp tiles of
//    split_tile non-zeros; tile partials combine per row in tile order.
//  * bounds: interleaved (lb, ub) pairs, current (read-only during a round) and
//    next (receives the FP64 min/max atomics); a bitmap records the variables
//    changed in the round.
//  * a row-contiguous copy of the SELL rows (xcol, xval): the deferred exact
//    pass reads rows that came from many slices, one row per lane (or group),
//    so it wants each row's elements next to each other; every row starts on
//    a 4-element boundary (zero padding), so a lane reads 4 columns or 2
//    coefficients with one 16-byte load.
//  * FP32 screen copies of the coefficients (sell_a32, la32) and of the
//    current bounds (bnd32): the screen streams 8 B per non-zero and gathers
//    8 B per bound pair; the FP64 arrays are read only by the exact pass.
//  * marking: per row position the round in which it must be processed next,
//    and the positions of every variable's rows (CSC of positions).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gdp_mlp.cuh"

namespace gdp {

// Partial activities of a split-row tile (and of a whole split row), with
// the first maximum of the FP64 |a| (ub - lb) over the tile's elements: km its
// bit pattern (never negative), p its element index within the row (-1: the
// leading 0.0 of the reference's maxactdelta).
struct TilePart {
    double minact, maxact;
    long long km;
    int minf, maxf;
    int p, pad;
};

// A row queued for the deferred exact pass: the index of its first element
// in the row-contiguous copy, its position and its length, so that the pass
// starts its element loads without looking the row up.
struct XRow {
    long long base;
    int pos, len;
    float slack_lo;  // the screen's lower bound of min(rhs - minact, maxact - lhs)
    int pad;
};

// FP32 screen partial of a split-row tile (see Scr in gdp_device.cuh).
struct TileScr {
    float mn, mx, S, U;
    int minf, maxf;
    int chg;  // a variable of the tile changed at the end of the previous round
    int pad;
};

// The FP32 screen copy of a variable's bounds (bnd_screen) with the round at
// whose end they were last committed (0: the input bounds), in one 16-byte
// record: the screen's gather of the bounds brings the stamp in the same sector.
// Batch members keep the 8-byte copies alone.
struct __align__(16) BndScr {
    float lb, ub;
    int round;
    int pad;
};

// Device-written round status. [0] is read by the host (CPU_LOOP), by the
// graph's condition kernel (GPU_LOOP) and by every CTA of the megakernel;
// [1], [2] are the megakernel's double-buffered per-round change flags.
struct RoundFlags {
    int change;          // a candidate tightened some bound in the (last) round
    int infeasible;      // the infeasibility rule fired
    int infeasible_var;  // smallest violating variable index (INT_MAX if none)
    int rounds;          // rounds executed
    int error;           // device-side error code (0 = none)
    int done;            // loop finished (GPU_LOOP / MEGAKERNEL)
    int mark_cur;        // this round processes only marked rows (else every row)
    unsigned tight;      // tightenings found in this round (decides the next round's mode)
    int exact;           // multi-tile rows of this round that need the exact pass
    int full_rounds;     // learned marking: rounds that swept every row
    int kind;            // learned marking, batched engine: kind of the round ([1 + parity])
    int infeasible_row;  // smallest row (original index) found infeasible (INT_MAX if none)
    unsigned long long changed_vars;  // committed variable changes, all rounds
    unsigned long long rows_proc;     // rows processed (screened), all rounds
    unsigned long long nnz_proc;      // their non-zeros
    unsigned long long nnz_exact;     // non-zeros that also went through the exact FP64 pass
    unsigned long long rows_deferred; // learned marking: marked rows the model left for a later round
    unsigned long long divisions;     // candidate divisions (bound candidates computed)
    unsigned long long rows_exact;    // SELL rows through the exact FP64 pass
    unsigned long long rows_go;       // ... of which had their candidates computed
    unsigned long long rows_seqmax;   // rows whose row test needed the sequential EPS-max (seq_eps_max)
    unsigned long long rows_drift;    // split rows skipped on their drift bound (counted once per row)
    unsigned long long nnz_drift;     // their non-zeros
};

enum DeviceError : int {
    kErrNone = 0,
    kErrBarrierTimeout = 1,  // a grid barrier wait exceeded its spin limit
    kErrQueueOverflow = 2,   // a batched work queue ran out of room (a bug: capacities are exact bounds)
};

// One entry of the marking index: a row position in which the variable
// appears and |a| of that element rounded up to FP32 (the drift bound's
// coefficient), in one 8-byte record so that placing an element scatters one
// store into the index.
struct alignas(8) VarEntry {
    int pos;
    float acoef;
};

struct DevProblem {
    int n;  // variables
    // thread rows
    int n_srows, n_slices;
    const long long *slice_ptr;  // n_slices + 1
    const int *slice_row0;       // n_slices + 1: first row position of each slice
    const int *slice_lg;         // n_slices: log2 of the lanes per row (SELL-g)
    const int *sell_col;
    const double *sell_val;
    const float *sell_a32;       // FP32 screen copies of sell_val (coef_screen)
    const int *srow_len;         // n_srows
    // row-contiguous copy of the SELL rows for the deferred exact pass: the
    // elements of position p at xptr[p] .. xptr[p] + srow_len[p] - 1
    const int *xptr;             // n_srows
    const int *xcol;
    const double *xval;
    const float *xa32;           // screen copies of xval
    const double *srow_lhs, *srow_rhs;
    // original row index of each position (SELL positions, then split rows)
    const int *pos_row;
    // split rows
    int n_lrows, n_tiles;
    const int *lcol;
    const double *lval;
    const float *la32;      // FP32 screen copies of lval
    const double *lrow_lhs, *lrow_rhs;
    const int *lrow_tile0;  // n_lrows + 1: tiles of split row r are [lrow_tile0[r], lrow_tile0[r+1])
    const int *tile_row;    // n_tiles
    const int *tile_begin;  // n_tiles (element offsets into lcol/lval)
    const int *tile_end;
    TilePart *tile_part;    // n_tiles: exact FP64 partials
    TileScr *tile_scr;      // n_tiles: FP32 screen partials
    int *row_exact;         // n_lrows: round in which the row needs the exact pass
    int n_mtiles;           // tiles of rows with more than one tile (candidate phase)
    const int *mtiles;
    // warp work items of the activity phase, heaviest first: s >= 0 is slice s,
    // s < 0 is split tile -s-1
    int n_items;
    const int *items;
    // marking (row positions: thread rows 0..n_srows-1, split rows n_srows + r).
    // use_marking: 0 never, 1 adaptive (a round runs on marked rows only when
    // the previous round found fewer than mark_threshold tightenings; pushing
    // marks costs about one write per non-zero of every changed variable), 2
    // always (tests).
    int use_marking;
    unsigned mark_threshold;
    // deferred exact pass (single-problem kernels): rows the FP32 screen
    // cannot skip are queued per lanes-per-row class (log2 g = 0..5) and run in
    // the next phase 32/g rows per warp, so the FP64 pipe sees full warps.
    // Class lg's queue is xrow[cls_begin[lg] .. cls_end[lg]) (its row positions
    // are exactly that range, slices being sorted by g).
    int defer_exact;
    int cls_begin[6], cls_end[6];
    XRow *xrow;            // n_srows
    unsigned *xctr;        // [parity * 16 + lg]: queue tails, [parity * 16 + 8 + lg]: pull counters
    // learned marking (SELL rows; null when no model is attached). learned:
    // 1 = rounds process the marked rows the model selects, 2 = trace (every
    // marked row is processed and logged with its label).
    int learned;
    float tau;             // logit threshold of the selection
    int learn_min_len;     // marked rows shorter than this are always processed
    MlpDev mlp;
    int *dirty;            // round since which the row has a changed variable (0: clean)
    int *dcount;           // variable changes in the row since it was last processed
    int *last_proc, *last_tight;  // last round the row was processed / tightened a bound
    float2 *rstat;         // last screen: normalised slack, log-ratio of U to the slack
    unsigned *rinfo;       // last screen: minf (2 bits), maxf (2 bits), exact (bit 4), go (bit 5), streak (bits 8..15)
    float *trace_x, *trace_y;  // trace: features (16 per sample) and labels
    unsigned *trace_n;
    unsigned trace_cap;
    int *mark;             // round in which the position is processed next (0: none)
    const int *pos_slice;  // n_srows: slice of each SELL row position
    // batched engine only (null otherwise): the round in which each slice was last queued
    int *slice_stamp;      // n_slices
    const int *var_ptr;    // n + 1
    const VarEntry *var_ent;  // var_ptr[j] .. var_ptr[j + 1] - 1: variable j's rows
    // drift bound of split rows (single-problem plain rounds): the certified
    // margin of the row's last screen skip (< 0: none), an upper bound of how
    // far its FP64 slack can have moved since (variables tightened), and the
    // round in which the screen skipped the row on that bound
    double *lrow_margin, *lrow_drift;
    int *lrow_skip;
    // bounds
    double2 *bnd;          // current (lb, ub); read-only while a round runs
    double2 *bnd_nxt;      // next: FP64 min/max atomics
    // FP32 screen copies of bnd, refreshed with it: BndScr records (bounds and
    // round stamp, 16 bytes) in single-problem contexts, float2 copies (8
    // bytes) in batch members
    float2 *bnd32;
    const unsigned char *is_cont;
    unsigned *chg;         // changed-variable bitmap, n_chg_words words
    int n_chg_words;
    RoundFlags *flags;
    unsigned *barrier;     // megakernel grid barrier {count, generation}
    unsigned *queue;       // work counters: [parity * 4 + phase]
    int max_rounds;
    long long spin_limit;  // clock64 cycles one grid-barrier wait may last (gdp_options.barrier_wait_kcycles)
};

constexpr int kWarpsPerCta = 8;
constexpr int kCtaThreads = 32 * kWarpsPerCta;

// Launch helpers (gdp_round.cu). All return the cudaError_t of the launch.
int launch_check_bounds(const DevProblem &P, int blocks, cudaStream_t s);
int launch_interleave(const DevProblem &P, const double *lb, const double *ub, int blocks, cudaStream_t s);
int launch_copy_out(const double *lb, const double *ub, double *lb_out, double *ub_out, int n, int blocks,
                    cudaStream_t s);
int launch_deinterleave(const DevProblem &P, double *lb, double *ub, int blocks, cudaStream_t s);
int launch_mark_all(const DevProblem &P, int blocks, cudaStream_t s);
int launch_round_begin(const DevProblem &P, cudaStream_t s);
int launch_activity_phase(const DevProblem &P, int blocks, cudaStream_t s);
int launch_candidate_phase(const DevProblem &P, int blocks, cudaStream_t s);
int launch_exact_phase(const DevProblem &P, int blocks, cudaStream_t s);
int launch_finalize(const DevProblem &P, int blocks, cudaStream_t s);
int launch_condition(const DevProblem &P, unsigned long long handle, cudaStream_t s);
// cta_warps: 4, 8 or 16 warps per CTA of the megakernel
int launch_megakernel(const DevProblem &P, int grid, int cta_warps, cudaStream_t s);
int phase_occupancy(int *act_blocks_per_sm, int *cand_blocks_per_sm, int *mega_blocks_per_sm, int cta_warps);
// Phase timers of the megakernel (a library built with GDP_PHASE_TIMERS):
// 0 or a CUDA error; -1 when the library was built without them.
int phase_timers_clear();
int phase_timers_read(unsigned long long *wall, unsigned long long *busy, unsigned long long *pass, int rounds);
// gdp_layout.cu: element arrays of the layout from the raw CSR (all device pointers)
struct LayoutBuild {
    const int *col, *row_ptr;  // raw CSR
    const double *val;
    int n_srows;
    const int *order;          // row position -> row
    const int *pos_slice, *slice_row0, *slice_lg, *xptr;
    const long long *slice_ptr;
    int *sell_col, *xcol;
    double *sell_val, *xval;
    float *sell_a32, *xa32;  // FP32 screen copies (coef_screen)
    int g1_begin;            // first position of the one-lane rows (n_srows: none)
    int n_lrows;
    const int *split_rows;     // split-row slot -> row
    const long long *lrow_ptr;
    int *lcol;
    double *lval;
    float *la32;
    // marking index, filled while the elements are placed: idx_cursor (n) hands
    // out each column's next slot of var_ent; columns out of range are skipped
    // (n: the variable count)
    int *idx_cursor;
    VarEntry *var_ent;
    int n;
    // row positions, built before the elements: SELL rows are sorted by
    // length, longest first, so the rows of one length L are the consecutive
    // positions from len_start[L] and their row-contiguous copies start at
    // len_base[L] + (p - len_start[L]) * L
    const double *lhs, *rhs;    // raw row sides (m)
    const int *len_start;       // lmax + 1 entries
    const long long *len_base;  // lmax + 1 entries
    int n_slices;
    int *srow_len_out, *xptr_out, *pos_slice_out;
    double *srow_lhs_out, *srow_rhs_out;
};
// Per row position: length, sides, first element of the row-contiguous copy
// and slice (the arrays that build_layout_elements reads as pos_slice, xptr).
int build_layout_positions(const LayoutBuild &L, int blocks, cudaStream_t s);
int build_layout_elements(const LayoutBuild &L, int blocks, cudaStream_t s);
// The first out-of-range column index (bad[0]) and the first non-finite
// coefficient (bad[1]) of the raw CSR, by atomicMin into bad, which the
// caller sets to INT_MAX before.
int check_csr_elements(const int *col, const double *val, int nnz, int n, int *bad, int blocks, cudaStream_t s);
// gdp_layout.cu: variable -> row-position index for marking (scratch: n + 2 + (n+1)/1024 ints)
// Column counts of the marking index from the raw CSR columns (out-of-range
// columns skipped): var_ptr (n + 1) gets their exclusive prefix sums and
// cursor (n + 1) a copy of it, from which the layout kernels hand out slots.
// scratch: (n + 1 + 1023) / 1024 + 1 ints.
int build_marking_counts(const int *col, int nnz, int n, int *var_ptr, int *cursor, int *scratch, cudaStream_t s);

}  // namespace gdp

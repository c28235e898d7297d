// gdp_internal.h -- device data layout shared by the host driver and kernels.
//
// HBM layout of one problem (built once per context, resident across rounds):
//  * thread rows (1 <= len <= thread_row_max): sorted by length, longest first,
//    grouped 32 to a slice; a slice stores its elements column-major
//    (element k of lane l at slice_ptr[s] + 32*k + l), so a warp streams a
//    slice with coalesced 128 B (col) / 256 B (val) loads while each lane sums
//    its own row left to right -- the reference's summation order.
//  * split rows (len > thread_row_max): CSR-contiguous, cut into tiles of
//    split_tile non-zeros; one CTA reduces a tile, partials combine per row in
//    tile order.
//  * bounds: cur (read-only during a round) and nxt (receives the FP64
//    min/max atomics); a bitmap records the variables changed in the round.
#pragma once

#include <cstdint>

namespace gdp {

struct RowActsPOD {
    double minact, maxact, maxactdelta;
    int minact_inf, maxact_inf;
};

// Device-written round status. Read by the host (CPU_LOOP), by the graph's
// conditional node (GPU_LOOP) and by every CTA of the megakernel.
struct RoundFlags {
    int change;          // a candidate tightened some bound in the (last) round
    int infeasible;      // the infeasibility rule fired
    int infeasible_var;  // smallest violating variable index (INT_MAX if none)
    int rounds;          // rounds executed
    int changed_vars;    // variables changed in the last round
    int error;           // device-side error code (0 = none)
    int done;            // loop finished (GPU_LOOP / MEGAKERNEL)
    int pad;
};

enum DeviceError : int {
    kErrNone = 0,
    kErrBarrierTimeout = 1,  // a grid barrier wait exceeded its spin limit
};

struct DevProblem {
    int n;                 // variables
    // thread rows
    int n_srows, n_slices;
    const long long *slice_ptr;  // n_slices + 1
    const int *sell_col;
    const double *sell_val;
    const int *srow_len;         // n_srows
    const double *srow_lhs, *srow_rhs;
    // split rows
    int n_lrows, n_tiles;
    const int *lcol;
    const double *lval;
    const double *lrow_lhs, *lrow_rhs;
    const int *lrow_tile0;       // n_lrows + 1: tiles of long row r are [lrow_tile0[r], lrow_tile0[r+1])
    const int *tile_row;         // n_tiles
    const int *tile_begin;       // n_tiles + 1 (element offsets; tile t = [tile_begin[t], tile_end[t]))
    const int *tile_end;
    RowActsPOD *tile_part;       // n_tiles
    // bounds
    double *lb, *ub;             // current (read-only while a round runs)
    double *lb_nxt, *ub_nxt;     // next (atomic min/max targets)
    const unsigned char *is_cont;
    unsigned *chg;               // changed-variable bitmap, n_chg_words words
    int n_chg_words;
    RoundFlags *flags;          // [0]: sticky state; [1], [2]: megakernel per-round change slots
    unsigned *barrier;          // megakernel grid barrier {count, generation}
    int max_rounds;
};

// Launch helpers (gdp_round.cu). All return the cudaError_t of the launch.
int launch_sell_round(const DevProblem &P, void *stream);
int launch_split_partial(const DevProblem &P, void *stream);
int launch_split_cand(const DevProblem &P, void *stream);
int launch_finalize(const DevProblem &P, int finalize_blocks, void *stream);
int launch_round_begin(const DevProblem &P, void *stream);
int launch_check_bounds(const DevProblem &P, int blocks, void *stream);
int launch_megakernel(const DevProblem &P, int grid, int block, void *stream);
int megakernel_occupancy(int block, int *blocks_per_sm);

constexpr int kSellWarpsPerCta = 8;
constexpr int kSplitThreads = 256;
constexpr int kFinalizeThreads = 256;
constexpr int kMegaThreads = 256;

}  // namespace gdp

/*
 * gdp_ext.h -- extended C API of the GB300 domain propagator (libgdp_gb300.so).
 *
 * The reference's C API (interface.h) uploads the problem, propagates and
 * frees everything in every call, and returns no round count or
 * infeasibility status. This header adds, with no counterpart in the
 * reference (so no reference citation applies to its entry points):
 *   - a persistent device context: upload a MIP once, propagate many bound
 *     vectors (branch-and-bound nodes) against it;
 *   - a stats struct (rounds, convergence, infeasibility, device time, bytes);
 *   - runtime options (round cap, loop driver, row-length thresholds) that the
 *     reference fixed at compile time (src/params.h).
 * Semantics of a propagation are those of interface.h: FP64 iterated
 * activity-based bound tightening to a fixpoint (reference
 * src/propagation_methods.cuh), run in deterministic Jacobi rounds.
 */
#ifndef GDP_GB300_EXT_H
#define GDP_GB300_EXT_H

#include <stddef.h>
#include "gdp_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gdp_context gdp_context; /* opaque */

typedef struct {
    int max_rounds;       /* round cap; <= 0 selects GDP_MAX_NUM_ROUNDS (100) */
    int sync_type;        /* GDP_SYNCTYPE: CPU_LOOP, GPU_LOOP or MEGAKERNEL */
    int thread_row_max;   /* rows up to this length run one lane per row (the reference's
                             left-to-right sums and row test, bit for bit); longer rows are
                             split into warp tiles. 0 selects the default (32). */
    int split_tile;       /* non-zeros per split-row warp tile; 0 selects the default (1024) */
    int device;           /* CUDA device ordinal (default 0) */
    int use_marking;      /* constraint marking: a round may process only the rows of variables
                             changed in the previous round (same result as sweeping every row).
                             1 (default, also -1): adaptive -- marked rounds follow rounds that
                             tightened fewer than n_vars/16 bounds; 0: always sweep every row;
                             2: every round after the first is marked */
    int ctas_per_sm;      /* resident CTAs per SM of the persistent round loop and of the phase
                             kernels; 0 (default) = as many as fit */
    int barrier_wait_kcycles; /* limit of one grid-barrier wait of the persistent loops (MEGAKERNEL,
                             learned marking, batches), in thousands of SM clock cycles; a CTA that
                             waits longer records a device error, every CTA leaves at its next
                             barrier and the call returns GDP_ERROR. 0 (default) = 4,000,000
                             (about 2 s at 2 GHz) */
    int cta_threads;      /* threads per CTA of the MEGAKERNEL loop: 128, 256 or 512; 0 (default) = 256.
                             With ctas_per_sm = 0 as many CTAs run per SM as fit (up to 6, 3 and 1,
                             about 24 warps per SM) */
    int reserved[4];      /* must be zero */
} gdp_options;

typedef struct {
    int rounds;             /* rounds executed (the reference's prop_round - 1) */
    int converged;          /* 1: the last round changed nothing (or infeasible) */
    int infeasible;         /* 1: some variable has lb - ub > GDP_FEASTOL*max(1,|lb|,|ub|), or some
                               row's activities exclude its sides: with no infinite contribution on
                               that side, minact - rhs or lhs - maxact > GDP_FEASTOL*max(1,|act|,|side|)
                               (the reference's isConsInfeasible with a relative tolerance) */
    int infeasible_var;     /* smallest violating variable, -1 if none */
    int device_error;       /* device-side error code, 0 if none */
    int kernel_launches;    /* kernels launched by the propagation */
    long long changed_vars; /* variable bound changes committed, summed over rounds */
    long long rows_processed;  /* rows swept, summed over rounds */
    long long nnz_processed;   /* their non-zeros */
    double bytes_algorithmic;  /* sum over rounds of 12*nnz + 20*rows + 36*n (CSR col+val,
                                  row_ptr+lhs+rhs, lb/ub read+write and vartype), rows and non-zeros
                                  counted as read: without those left unread on their drift bound */
    double device_ms;       /* device time of the round loop (CUDA events) */
    double total_ms;        /* host wall time of the call */
    long long nnz_exact;    /* non-zeros of the rows that the FP32 screen could not skip and that
                               went through the exact FP64 pass, summed over rounds */
    long long rows_deferred; /* learned marking: marked rows the model left for a later round */
    int full_rounds;        /* learned marking: rounds that swept every row (incl. the certification) */
    int infeasible_row;     /* smallest row found infeasible by the row rule, -1 if none */
    long long divisions;    /* bound candidates computed (one FP64 division each), summed over rounds */
    long long rows_exact;   /* rows up to split_tile non-zeros that went through the exact FP64 pass */
    long long rows_go;      /* ... of which passed the row test (candidates computed) */
    long long rows_seqmax;  /* row tests that needed the reference's sequential EPS-max of |a|(ub-lb)
                               (the FP64 maximum exceeded the slack by EPS to 2.00001e-9) */
    long long rows_drift;   /* marked split rows (longer than split_tile) left unread because their
                               last screen's certified margin still covers every tightening of their
                               variables since (counted in rows_processed / nnz_processed as screened) */
    long long nnz_drift;    /* their non-zeros */
} gdp_stats;

/* Fills *opts with the defaults. */
GDP_RETCODE gdp_default_options(gdp_options *opts);

/* Last error message of the calling thread ("" if none). */
const char *gdp_last_error(void);

/* Device memory released by destroyed contexts and batches stays cached (up
 * to 32 GiB) for later contexts of similar size, so that repeated
 * create / destroy cycles allocate nothing; a failed allocation frees the
 * cache and retries. This frees the cache now. */
GDP_RETCODE gdp_release_cached_memory(void);

/* Uploads a MIP (host CSR arrays, reference argument meaning) and builds the
 * device layout. opts may be NULL. The context owns its device memory and a
 * CUDA stream; it is not thread-safe (use one context per thread). */
GDP_RETCODE gdp_context_create(int n_cons, int n_vars, int nnz, const int *csr_col_indices,
                               const int *csr_row_ptrs, const double *csr_vals,
                               const double *lhss, const double *rhss, const int *vartypes,
                               const gdp_options *opts, gdp_context **out);

GDP_RETCODE gdp_context_destroy(gdp_context *ctx);

/* Propagates host bounds lbs/ubs (n_vars each, in/out) to a fixpoint.
 * stats may be NULL. */
GDP_RETCODE gdp_propagate(gdp_context *ctx, double *lbs, double *ubs, gdp_stats *stats);

/* As gdp_propagate, with the bounds read from lbs_in/ubs_in and the fixpoint
 * written to lbs_out/ubs_out (n_vars each; an output may be its input). The
 * inputs are copied to the outputs first (host threads), so on error the
 * outputs hold the inputs. */
GDP_RETCODE gdp_propagate_into(gdp_context *ctx, const double *lbs_in, const double *ubs_in, double *lbs_out,
                               double *ubs_out, gdp_stats *stats);

/* Same on device-resident bounds (d_lbs/d_ubs: n_vars doubles each in device
 * memory, in/out) on the given CUDA stream (NULL: the context's stream). The
 * call returns after the propagation has finished. */
GDP_RETCODE gdp_propagate_device(gdp_context *ctx, double *d_lbs, double *d_ubs, void *stream,
                                 gdp_stats *stats);

/* Changes the round cap / driver of an existing context. */
GDP_RETCODE gdp_context_set_options(gdp_context *ctx, int max_rounds, int sync_type);

/* Layout facts of a context: number of thread rows, slices, split rows and
 * split tiles, padded SELL elements (for tests and tuning). */
GDP_RETCODE gdp_context_layout(const gdp_context *ctx, long long out[6]);

/* The C API call of interface.h with options and stats. */
GDP_RETCODE gdp_propagate_once(int n_cons, int n_vars, int nnz, const int *csr_col_indices,
                               const int *csr_row_ptrs, const double *csr_vals,
                               const double *lhss, const double *rhss, double *lbs, double *ubs,
                               const int *vartypes, const gdp_options *opts, gdp_stats *stats);

/* ---- batched propagation (no counterpart in the reference, which
 * propagates one problem per call) ----------------------------------------
 * A batch propagates many problems ("instances"), or many bound vectors of one
 * context's problem ("nodes", e.g. branch-and-bound children), together in
 * one persistent cooperative launch that is captured once into a CUDA graph
 * and replayed. Every member gets the bounds, round count and infeasibility
 * verdict that a single-problem propagation of it returns; members that
 * converge early stop costing work. */
typedef struct gdp_batch gdp_batch;

/* Instances: per-instance host arrays with the reference's CSR meaning.
 * opts (may be NULL) applies to every instance. */
GDP_RETCODE gdp_batch_create(int n_inst, const int *n_cons, const int *n_vars, const int *nnz,
                             const int *const *csr_col_indices, const int *const *csr_row_ptrs,
                             const double *const *csr_vals, const double *const *lhss,
                             const double *const *rhss, const int *const *vartypes,
                             const gdp_options *opts, gdp_batch **out);

/* Nodes of ctx's problem (ctx must outlive the batch). When ctx's last
 * propagation converged feasibly, round 1 of every node processes only the
 * rows of the variables whose bounds differ from that fixpoint (the other rows
 * are at their fixpoint already); otherwise round 1 processes every row. */
GDP_RETCODE gdp_batch_create_nodes(gdp_context *ctx, int n_nodes, gdp_batch **out);

/* lbs[k], ubs[k]: member k's bounds (host, in/out, n_vars of member k).
 * member_stats: one entry per member, or NULL; total: batch sums (rounds = the
 * largest member round count, device_ms = the whole launch), or NULL. */
GDP_RETCODE gdp_batch_propagate(gdp_batch *b, double *const *lbs, double *const *ubs,
                                gdp_stats *member_stats, gdp_stats *total);

/* As gdp_batch_propagate, with member k's bounds read from lbs_in[k] /
 * ubs_in[k] and its fixpoint written to lbs_out[k] / ubs_out[k] (an output
 * may be its input); the outputs are written only when the call succeeds. */
GDP_RETCODE gdp_batch_propagate_into(gdp_batch *b, const double *const *lbs_in, const double *const *ubs_in,
                                     double *const *lbs_out, double *const *ubs_out, gdp_stats *member_stats,
                                     gdp_stats *total);

/* 1 if the batch runs as a captured CUDA graph (known after the first
 * propagation), 0 if it launches the same sequence directly. */
int gdp_batch_uses_graph(const gdp_batch *b);

GDP_RETCODE gdp_batch_destroy(gdp_batch *b);

/* ---- learned row marking (no counterpart in the reference) ------------------
 * A 16 -> 64 -> 64 -> 1 MLP (ReLU; BF16 weights and activations, FP32
 * accumulation; forward and the activation-gradient product on the tensor
 * cores) scores, from per-row features, whether processing a row that a
 * changed variable marked will tighten a bound. Parameters are one FP32
 * vector of GDP_MLP_PARAMS floats: W1[64][16], b1[64], W2[64][64], b2[64],
 * w3[64], b3. Features are GDP_MLP_FEATURES floats per row (see
 * gdp_context_trace). */
#define GDP_MLP_FEATURES 16
#define GDP_MLP_PARAMS 5313
typedef struct gdp_mlp gdp_mlp;

/* He-uniform weights from `seed`, zero biases, on `device`. */
GDP_RETCODE gdp_mlp_create(unsigned long long seed, int device, gdp_mlp **out);
GDP_RETCODE gdp_mlp_destroy(gdp_mlp *m);
GDP_RETCODE gdp_mlp_get_params(const gdp_mlp *m, float *params);
/* Sets the FP32 master parameters (and resets the optimizer state). */
GDP_RETCODE gdp_mlp_set_params(gdp_mlp *m, const float *params);
/* logits[i] of the n x 16 host features x (rounded to BF16 on the device). */
GDP_RETCODE gdp_mlp_forward(gdp_mlp *m, int n, const float *x, float *logits);
/* Gradient (GDP_MLP_PARAMS floats) and value of the weighted binary
 * cross-entropy sum_i w_i BCE(sigmoid(z_i), y_i) / sum_i w_i at the current
 * parameters. */
GDP_RETCODE gdp_mlp_gradient(gdp_mlp *m, int n, const float *x, const float *y, const float *w, float *grad,
                             float *loss);
/* Adam (beta 0.9 / 0.999) over minibatches of `batch` samples for `epochs`
 * passes, on the device; final_loss (may be NULL): the last epoch's mean loss. */
GDP_RETCODE gdp_mlp_train(gdp_mlp *m, int n, const float *x, const float *y, const float *w, int epochs,
                          int batch, float lr, unsigned long long seed, float *final_loss);

/* Attaches `model` (NULL detaches) to ctx: its propagations then run learned
 * rounds. A learned round processes the marked rows (rows with a variable
 * changed since they were last processed) whose logit is >= threshold, plus
 * every marked row shorter than min_len non-zeros; the others stay marked for a
 * later round. Rows longer than split_tile are always processed when marked. A
 * learned round that changes nothing is followed by a round over every marked
 * row, one of those that changes nothing by a round over every row, and the
 * propagation ends only when such a full round changes nothing (or at
 * max_rounds), so the bounds are a certified fixpoint whatever the model
 * predicts. The model must outlive its use by ctx; learned propagations always
 * run as one persistent launch. */
GDP_RETCODE gdp_context_set_model(gdp_context *ctx, const gdp_mlp *model, float threshold, int min_len);

/* Learned row marking for every member of an instance batch (model NULL: off):
 * each member runs the rounds gdp_context_set_model describes -- its own
 * sequence of learned, flush and full rounds, ended by a full round that
 * changes nothing -- inside the batch's one persistent launch, with the
 * bounds, round count and verdict of its single-problem learned propagation.
 * Node batches return GDP_ERROR. The model must outlive its use by b. */
GDP_RETCODE gdp_batch_set_model(gdp_batch *b, const gdp_mlp *model, float threshold, int min_len);

/* Trace propagation of ctx's problem from lbs/ubs (host, in/out) with exact
 * marking (every marked row processed): for each marked row of a marked round
 * the 16 features before processing go to features[16 * i ..] and the label
 * (1: processing it tightened a bound) to labels[i], for the first `capacity`
 * such rows; *n_samples receives their count. Features: log2(1+len)/16;
 * last screen's infinity counts minf/3, maxf/3 (capped at 3); normalised slack
 * and log-ratio of the activity-delta bound to the slack; lhs infinite; rhs
 * infinite; equality row; rounds since the row last tightened, was last
 * processed, and has been marked (each min(.,63)/63); changed variables since
 * last processed / len; unproductive-processing streak/15; last screen said
 * exact; last row test said go; never processed. */
GDP_RETCODE gdp_context_trace(gdp_context *ctx, double *lbs, double *ubs, int capacity, float *features,
                              float *labels, int *n_samples, gdp_stats *stats);

/* ---- autotuner (no counterpart in the reference) ---------------------------
 * Times the propagation of one problem from lbs/ubs (host, not modified) in
 * two stages, `repeats` times per candidate (best device time counts),
 * starting from `base` (may be NULL) for every other option: first the row
 * bins (thread_row_max in {16, 32, 64} x split_tile in {512, 1024, 2048})
 * under base's schedule (MEGAKERNEL if base's is CPU_LOOP), then, on the
 * fastest bins, the loop schedule: MEGAKERNEL with 128-, 256- or 512-thread
 * CTAs at several CTAs per SM, and GPU_LOOP. *best receives the fastest
 * options and *best_ms their device time; trials (may be NULL) receives up
 * to max_trials records and *n_trials their count. The layouts only change
 * the summation order of rows longer than thread_row_max (each layout is
 * bit-exact with the oracle's matching GPU mode), so on slowly converging
 * continuous bounds the round count may differ by a round between
 * candidates; the time to the fixpoint is what counts.
 * Results are cached per problem shape (device, m, n, nnz, the histogram of
 * row lengths in powers of two, base's round cap and marking): a later call
 * for a problem of the same shape returns the cached options and trials at
 * once. gdp_autotune_clear_cache empties the cache. */
typedef struct {
    int thread_row_max, split_tile, sync_type, ctas_per_sm, rounds, cta_threads;
    double ms;
} gdp_tune_trial;
GDP_RETCODE gdp_autotune(int n_cons, int n_vars, int nnz, const int *csr_col_indices, const int *csr_row_ptrs,
                         const double *csr_vals, const double *lhss, const double *rhss, const double *lbs,
                         const double *ubs, const int *vartypes, const gdp_options *base, int repeats,
                         gdp_options *best, double *best_ms, gdp_tune_trial *trials, int max_trials,
                         int *n_trials);
GDP_RETCODE gdp_autotune_clear_cache(void);

/* ---- phase timers (no counterpart in the reference) ----------------------
 * Where a MEGAKERNEL propagation spends its time, from a library built with
 * GDP_PHASE_TIMERS (build.py --phase-timers, libgdp_gb300_timers.so; the plain
 * library returns GDP_NOTIMPLEMENTED). Per round r (0 <= r < rounds, at most
 * 1024; round numbers start at 1), 8 values each:
 *   wall[8r + k]: %globaltimer ns at the round's start (k = 0) and after the
 *     grid barriers of phase A (1), B (2), C (3, rounds with exact tiles) and
 *     F (4); k = 5..7: rows, non-zeros and exact non-zeros processed so far;
 *   busy[8r + k]: warp ns summed over all warps in phase A (0), B multi-tile
 *     rows (1), B deferred exact rows (2), C (3), F (4); k = 5..7: the longest
 *     time of one warp in one of A (5), B's two parts (6), C or F (7);
 *   pass[2 lg + i] (16 values, all rounds): warp ns of the exact pass of rows
 *     summed by 2^lg lanes, pass 1 (i = 0, activities and row test) and pass 2
 *     (i = 1, candidates); pass[12]: elements of the one-lane rows through the
 *     exact pass, pass[13]: 32 x the longest such row of each warp, summed.
 * Any output may be NULL. The timers accumulate over propagations until
 * gdp_phase_timers_clear; they are device globals of the current device. */
GDP_RETCODE gdp_phase_timers_clear(void);
GDP_RETCODE gdp_phase_timers_read(unsigned long long *wall, unsigned long long *busy, unsigned long long *pass,
                                  int rounds);

/* ---- MPS reader (no counterpart in the reference, which reads MPS through
 * python-mip, fileReader/readerInterface.py:52-145) ---------------------------
 * Parses free-format MPS text (decompress .gz first) into the reference's CSR
 * convention: constraint rows in ROWS order (objective rows dropped), entries
 * of a row in column order, lhs/rhs with infinite sides as +-inf, bounds
 * (default [0, +inf); UP < 0 with an untouched lower bound 0 gives lb = -inf),
 * RANGES per the MPS standard, SCIP variable types (integer from MARKER
 * INTORG/INTEND blocks or LI/UI/BV bounds; integer with bounds [0, 1] is
 * binary). The arrays are malloc'ed by the library; release them with
 * gdp_mps_free. */
typedef struct {
    int n_cons, n_vars, nnz;
    int *row_ptr, *col;
    double *val, *lhs, *rhs, *lb, *ub;
    int *vartype;
} gdp_mps_problem;
GDP_RETCODE gdp_mps_parse(const char *text, long long len, gdp_mps_problem *out);
void gdp_mps_free(gdp_mps_problem *p);

/* Propagation that allocates no memory, for callers that cannot call
 * cudaMalloc (e.g. a solver or framework whose device memory belongs to its
 * own pool and that propagates many nodes in a loop, where cudaMalloc/cudaFree
 * would synchronize the device and fragment that pool). No counterpart in the
 * reference.
 *   - Every array argument is DEVICE memory (CSR with the reference's meaning,
 *     bounds in/out); nothing is copied to or from the host except the round
 *     flags.
 *   - Working memory is one fixed device array inside the library, sized for
 *     GDP_NOALLOC_MAX_VARS variables (about 16 MiB); every GPU that loads the
 *     library holds it until the process exits. n_vars above the limit returns
 *     GDP_ERROR.
 *   - The first call on a device looks up that array's device address (once per
 *     device).
 *   - The host reads the round flags after every round: the call synchronizes
 *     its stream once per round.
 *   - Calls share the array: calls that overlap on the GPU race and must be
 *     serialized by the caller. Each call re-initializes it.
 *   - Rows are summed left to right by one thread each: results equal the
 *     context path's for rows up to its thread_row_max non-zeros.
 * stream: CUDA stream (NULL = legacy default stream); the call returns when the
 * propagation has finished. stats may be NULL (device_ms is not measured). */
#define GDP_NOALLOC_MAX_VARS (1 << 20)
GDP_RETCODE gdp_propagate_noalloc(int n_cons, int n_vars, int nnz, const int *d_csr_col_indices,
                                  const int *d_csr_row_ptrs, const double *d_csr_vals,
                                  const double *d_lhss, const double *d_rhss, double *d_lbs,
                                  double *d_ubs, const int *d_vartypes, int max_rounds, void *stream,
                                  gdp_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* GDP_GB300_EXT_H */

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
    int reserved[7];      /* must be zero */
} gdp_options;

typedef struct {
    int rounds;             /* rounds executed (the reference's prop_round - 1) */
    int converged;          /* 1: the last round changed nothing (or infeasible) */
    int infeasible;         /* 1: some variable has lb - ub > GDP_FEASTOL*max(1,|lb|,|ub|) */
    int infeasible_var;     /* smallest violating variable, -1 if feasible */
    int device_error;       /* device-side error code, 0 if none */
    int kernel_launches;    /* kernels launched by the propagation */
    long long changed_vars; /* variable bound changes committed, summed over rounds */
    long long rows_processed;  /* rows swept, summed over rounds */
    long long nnz_processed;   /* their non-zeros */
    double bytes_algorithmic;  /* sum over rounds of 12*nnz + 20*rows + 36*n
                                  (CSR col+val, row_ptr+lhs+rhs, lb/ub read+write and vartype) */
    double device_ms;       /* device time of the round loop (CUDA events) */
    double total_ms;        /* host wall time of the call */
    long long nnz_exact;    /* non-zeros of the rows that the FP32 screen could not skip and that
                               went through the exact FP64 pass, summed over rounds */
} gdp_stats;

/* Fills *opts with the defaults. */
GDP_RETCODE gdp_default_options(gdp_options *opts);

/* Last error message of the calling thread ("" if none). */
const char *gdp_last_error(void);

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

/* 1 if the batch runs as a captured CUDA graph (known after the first
 * propagation), 0 if it launches the same sequence directly. */
int gdp_batch_uses_graph(const gdp_batch *b);

GDP_RETCODE gdp_batch_destroy(gdp_batch *b);

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
 *     device); make that first call before any stream capture.
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

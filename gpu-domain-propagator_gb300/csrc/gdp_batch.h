// gdp_batch.h -- host side of the batched engine (gdp_batch.cu).
#pragma once

#include <memory>
#include <vector>

#include "gdp_context.h"

namespace gdp {

// Kernel-side view of a batch.
struct BatchDev {
    DevProblem *units;  // n_units
    int n_units;
    const int *wbase;   // n_units + 1: first change-bitmap word of each unit in the batch's word space
    int total_words;
    int max_rounds;
    unsigned long long *entries;  // 2 x cap_entries: (unit << 32 | work item) queued for a round, by parity
    unsigned cap_entries;
    unsigned long long *cq, *xq;  // tiles of multi-tile rows: candidate-phase / exact-phase queues
    unsigned cap_tiles;
    unsigned *ctr;        // work counters [parity * 4 + phase]
    unsigned *tail;       // [0], [1]: entries by parity; [2]: cq; [3]: xq
    int *fs_unit;         // units swept in full in the coming round
    int *fs_prefix;       // n_fs + 1: prefix of their work-item counts
    int *n_fs;
    unsigned *barrier;    // {count, generation}
    int *error;
    int *rounds_out;
    int *n_pending;       // learned units that need the next round (learned batches)
    long long spin_limit; // clock64 cycles one grid-barrier wait may last (the first member's option)
};

int launch_batch(const BatchDev &B, int grid, const double *lb, const double *ub, double *lb_out,
                 double *ub_out, const long long *var_base, int max_unit_n, const double2 *ref,
                 const int *seed_mode, bool learned, cudaStream_t s);
int batch_occupancy(int *blocks_per_sm, bool learned);

class Batch {
public:
    ~Batch();
    // Distinct problems, one unit each (host CSR arrays).
    GDP_RETCODE init_instances(int n_inst, const int *n_cons, const int *n_vars, const int *nnz,
                               const int *const *col, const int *const *row_ptr, const double *const *val,
                               const double *const *lhs, const double *const *rhs, const int *const *vartype,
                               const gdp_options *o);
    // n_nodes bound vectors of ctx's problem (the context must outlive the batch).
    GDP_RETCODE init_nodes(Context *ctx, int n_nodes);
    // lbs[k], ubs[k]: member k's bounds (host, in/out).
    // Member k's bounds are read from lbs_in[k] / ubs_in[k] and its fixpoint
    // written to lbs_out[k] / ubs_out[k] (an output may be its input).
    GDP_RETCODE propagate(const double *const *lbs_in, const double *const *ubs_in, double *const *lbs_out,
                          double *const *ubs_out, gdp_stats *member_stats, gdp_stats *total);
    // Instance batches: learned row marking for every member (m == nullptr: off).
    GDP_RETCODE set_model(const Mlp *m, float threshold, int min_len);

    int n_units = 0;
    bool nodes = false;
    bool use_graph = true;   // capture the device part once and replay it
    bool graph_ok = false;   // the graph was captured and is used
    int grid = 1;
    int max_rounds = GDP_MAX_NUM_ROUNDS;

private:
    GDP_RETCODE finish_init(int device, int ctas_per_sm);
    GDP_RETCODE size_grid();
    GDP_RETCODE enqueue(cudaStream_t s);
    void copy_in(const double *const *lbs, const double *const *ubs);
    void copy_out(double *const *lbs, double *const *ubs);

    std::vector<std::unique_ptr<Context>> inst_;  // instances (units in heaviest-first order)
    Context *base_ = nullptr;                     // nodes
    std::vector<int> member_of_unit_;             // unit -> member index of the caller
    bool learned_ = false;                        // members run learned rounds (set_model)
    int device_ = 0, ctas_per_sm_ = 0;
    std::vector<DevProblem> units_h_;
    std::vector<long long> var_base_;             // unit -> first variable in the staging buffers
    long long total_vars_ = 0;
    int max_unit_n_ = 0;
    Arena arena_;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    BatchDev B_{};
    double *h_lb_ = nullptr, *h_ub_ = nullptr;  // pinned staging
    double *d_lb_ = nullptr, *d_ub_ = nullptr;
    long long *d_var_base_ = nullptr;
    int *d_seed_mode_ = nullptr;
    std::vector<int> seed_mode_;                // 0: round 1 sweeps every row; 1: marks from ref
    const double2 *ref_ = nullptr;              // certified fixpoint (nodes)
    RoundFlags *h_flags_ = nullptr;             // pinned: n_units x 3, device result
    RoundFlags *h_flags_init_ = nullptr;        // pinned: initial values
    RoundFlags *d_flags_ = nullptr;
    int *h_rounds_ = nullptr;                   // pinned: {error, rounds}
    int *h_seed_ = nullptr;                     // pinned: per-unit seed mode of this call
    bool graph_failed_ = false;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
};

}  // namespace gdp

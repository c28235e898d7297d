// gdp_context.h -- host-side propagation context (device layout + drivers).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gdp_ext.h"
#include "gdp_internal.h"
#include "gdp_mlp.h"

namespace gdp {

void set_error(const std::string &msg);
const char *last_error();

// Owns device allocations. Released blocks go to a process-wide cache of
// device memory that later arenas draw from, so contexts of one problem size
// can be created and destroyed without cudaMalloc / cudaFree (each costs up
// to milliseconds for blocks of hundreds of MB).
struct Arena {
    struct Block {
        void *p;
        size_t bytes;
        int dev;
    };
    std::vector<Block> blocks;
    ~Arena();
    void *alloc_bytes(size_t bytes);
    void release();  // waits for the device, then returns every block to the cache
};

// Frees the cached device memory of released arenas (all devices).
void release_cached_memory();

GDP_RETCODE autotune(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                     const double *lhs, const double *rhs, const double *lbs, const double *ubs,
                     const int *vartype, const gdp_options *base, int repeats, gdp_options *best,
                     double *best_ms, gdp_tune_trial *trials, int max_trials, int *n_trials);
GDP_RETCODE autotune_clear_cache();

GDP_RETCODE validate_csr(int m, int n, int nnz, const int *col, const int *row_ptr,
                         const double *val, const int *vartype);

class Context {
public:
    ~Context();
    GDP_RETCODE init(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                     const double *lhs, const double *rhs, const int *vartype, const gdp_options *o);
    GDP_RETCODE propagate_host(double *lbs, double *ubs, gdp_stats *st);
    GDP_RETCODE propagate_device(double *d_lbs, double *d_ubs, cudaStream_t s, gdp_stats *st);
    // Loop driver, resident CTAs per SM (0: as many as fit) and megakernel CTA
    // size of later propagations; the layout stays.
    GDP_RETCODE set_schedule(int sync_type, int ctas_per_sm, int cta_threads);
    // Learned marking with model m (NULL: off), logit threshold and the
    // shortest row length the model decides for.
    GDP_RETCODE set_model(const Mlp *m, float threshold, int min_len);
    // Trace propagation: exact marking, logging up to `capacity` samples.
    GDP_RETCODE trace(double *lbs, double *ubs, int capacity, float *x_out, float *y_out, int *n_out,
                      gdp_stats *st);

    int m = 0, n = 0, nnz = 0;
    gdp_options opts{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    RoundFlags *h_flags = nullptr;  // pinned
    Arena arena;
    DevProblem P{};
    double *d_lb = nullptr, *d_ub = nullptr;  // staging for host bounds
    int n_sms = 0, vec_blocks = 1, act_blocks = 1, cand_blocks = 1, mega_grid = 1, learned_grid = 1;
    int mega_warps = 8;  // warps per CTA of the megakernel (opts.cta_threads / 32)
    int n_srows = 0, n_slices = 0, n_lrows = 0, n_tiles = 0;
    long long sell_elems = 0;
    // the last propagation converged feasibly: P.bnd is a fixpoint of the problem
    bool certified = false;
    bool host_direct = false;  // kernels read and write pageable host memory (coherent access)
    // GPU_LOOP graph (built on first use, reused while the context lives)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;

private:
    GDP_RETCODE run(const double *lb_in, const double *ub_in, double *lb_out, double *ub_out,
                    cudaStream_t s, gdp_stats *st);
    GDP_RETCODE build_graph(cudaStream_t s);
    GDP_RETCODE rounds_cpu_loop(cudaStream_t s, int *launches);
    GDP_RETCODE rounds_gpu_loop(cudaStream_t s, int *launches);
    GDP_RETCODE rounds_megakernel(cudaStream_t s, int *launches);
    GDP_RETCODE rounds_learned(cudaStream_t s, int *launches);
    GDP_RETCODE alloc_learned_state();
};

}  // namespace gdp

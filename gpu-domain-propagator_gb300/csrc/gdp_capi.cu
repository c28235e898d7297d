// gdp_capi.cu -- the extern "C" surface of libgdp_gb300.so: the reference's
// interface.h symbols (include/interface.h of the reference, implemented in
// its src/interface.cu:18-354) and the extended API of gdp_ext.h.
#include <chrono>
#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "gdp_batch.h"
#include "gdp_context.h"
#include "gdp_mlp.h"
#include "interface.h"

using gdp::Context;

struct gdp_context {
    Context impl;
};

struct gdp_batch {
    gdp::Batch impl;
};

namespace {

// The reference's CALL_AND_HANDLE (src/interface.cu:7-16): exceptions become
// GDP_ERROR; here with the message kept for gdp_last_error().
template <class F>
GDP_RETCODE guarded(F &&f) {
    try {
        return f();
    } catch (const std::bad_alloc &) {
        gdp::set_error("host allocation failed");
        return GDP_ERROR;
    } catch (const std::exception &e) {
        gdp::set_error(e.what());
        return GDP_ERROR;
    } catch (...) {
        gdp::set_error("unknown exception");
        return GDP_ERROR;
    }
}

GDP_RETCODE propagate_once_impl(int n_cons, int n_vars, int nnz, const int *col, const int *row_ptr,
                                const double *val, const double *lhs, const double *rhs,
                                double *lbs, double *ubs, const int *vartypes,
                                const gdp_options *opts, gdp_stats *stats) {
    const auto t0 = std::chrono::steady_clock::now();
    if (stats) *stats = gdp_stats{};
    // reference GPU_propagator.cuh:113-116: empty problems are a no-op
    if (n_cons == 0 || n_vars == 0 || nnz == 0) {
        if (stats) { stats->converged = 1; stats->infeasible_var = -1; stats->infeasible_row = -1; }
        return GDP_OKAY;
    }
    if (!lbs || !ubs) { gdp::set_error("null lbs/ubs"); return GDP_ERROR; }
    Context ctx;
    GDP_RETCODE rc = ctx.init(n_cons, n_vars, nnz, col, row_ptr, val, lhs, rhs, vartypes, opts);
    if (rc != GDP_OKAY) return rc;
    rc = ctx.propagate_host(lbs, ubs, stats);
    if (stats)
        stats->total_ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

}  // namespace

// Only the C API is exported (the library builds with -fvisibility=hidden).
#pragma GCC visibility push(default)
extern "C" {

GDP_RETCODE gdp_default_options(gdp_options *o) {
    if (!o) return GDP_ERROR;
    *o = gdp_options{};
    o->max_rounds = GDP_MAX_NUM_ROUNDS;
    o->sync_type = CPU_LOOP;
    o->thread_row_max = 32;
    o->split_tile = 1024;
    o->device = 0;
    o->use_marking = 1;
    return GDP_OKAY;
}

const char *gdp_last_error(void) { return gdp::last_error(); }

GDP_RETCODE gdp_release_cached_memory(void) {
    return guarded([&]() -> GDP_RETCODE {
        gdp::release_cached_memory();
        return GDP_OKAY;
    });
}

GDP_RETCODE gdp_context_create(int n_cons, int n_vars, int nnz, const int *col, const int *row_ptr,
                               const double *val, const double *lhs, const double *rhs,
                               const int *vartypes, const gdp_options *opts, gdp_context **out) {
    return guarded([&]() -> GDP_RETCODE {
        if (!out) { gdp::set_error("null output pointer"); return GDP_ERROR; }
        *out = nullptr;
        if (n_cons <= 0 || n_vars <= 0 || nnz <= 0) {
            gdp::set_error("a context needs n_cons, n_vars and nnz > 0");
            return GDP_ERROR;
        }
        gdp_context *c = new gdp_context();
        const GDP_RETCODE rc = c->impl.init(n_cons, n_vars, nnz, col, row_ptr, val, lhs, rhs, vartypes, opts);
        if (rc != GDP_OKAY) { delete c; return rc; }
        *out = c;
        return GDP_OKAY;
    });
}

GDP_RETCODE gdp_batch_create(int n_inst, const int *n_cons, const int *n_vars, const int *nnz,
                             const int *const *col, const int *const *row_ptr, const double *const *val,
                             const double *const *lhs, const double *const *rhs, const int *const *vartypes,
                             const gdp_options *opts, gdp_batch **out) {
    return guarded([&]() -> GDP_RETCODE {
        if (!out) { gdp::set_error("null output pointer"); return GDP_ERROR; }
        *out = nullptr;
        if (n_inst <= 0 || !n_cons || !n_vars || !nnz || !col || !row_ptr || !val || !lhs || !rhs || !vartypes) {
            gdp::set_error("a batch needs n_inst > 0 and every per-instance array");
            return GDP_ERROR;
        }
        for (int k = 0; k < n_inst; k++)
            if (n_cons[k] <= 0 || n_vars[k] <= 0 || nnz[k] <= 0) {
                gdp::set_error("instance " + std::to_string(k) + " needs n_cons, n_vars and nnz > 0");
                return GDP_ERROR;
            }
        gdp_batch *b = new gdp_batch();
        const GDP_RETCODE rc =
            b->impl.init_instances(n_inst, n_cons, n_vars, nnz, col, row_ptr, val, lhs, rhs, vartypes, opts);
        if (rc != GDP_OKAY) { delete b; return rc; }
        *out = b;
        return GDP_OKAY;
    });
}

GDP_RETCODE gdp_batch_create_nodes(gdp_context *ctx, int n_nodes, gdp_batch **out) {
    return guarded([&]() -> GDP_RETCODE {
        if (!out) { gdp::set_error("null output pointer"); return GDP_ERROR; }
        *out = nullptr;
        if (!ctx) { gdp::set_error("null context"); return GDP_ERROR; }
        gdp_batch *b = new gdp_batch();
        const GDP_RETCODE rc = b->impl.init_nodes(&ctx->impl, n_nodes);
        if (rc != GDP_OKAY) { delete b; return rc; }
        *out = b;
        return GDP_OKAY;
    });
}

GDP_RETCODE gdp_batch_propagate(gdp_batch *b, double *const *lbs, double *const *ubs, gdp_stats *member_stats,
                                gdp_stats *total) {
    return guarded([&]() -> GDP_RETCODE {
        if (!b) { gdp::set_error("null batch"); return GDP_ERROR; }
        return b->impl.propagate(lbs, ubs, lbs, ubs, member_stats, total);
    });
}

GDP_RETCODE gdp_batch_propagate_into(gdp_batch *b, const double *const *lbs_in, const double *const *ubs_in,
                                     double *const *lbs_out, double *const *ubs_out, gdp_stats *member_stats,
                                     gdp_stats *total) {
    return guarded([&]() -> GDP_RETCODE {
        if (!b) { gdp::set_error("null batch"); return GDP_ERROR; }
        return b->impl.propagate(lbs_in, ubs_in, lbs_out, ubs_out, member_stats, total);
    });
}

int gdp_batch_uses_graph(const gdp_batch *b) { return b && b->impl.graph_ok ? 1 : 0; }

GDP_RETCODE gdp_batch_destroy(gdp_batch *b) {
    return guarded([&]() -> GDP_RETCODE {
        delete b;
        return GDP_OKAY;
    });
}

GDP_RETCODE gdp_context_set_model(gdp_context *ctx, const gdp_mlp *model, float threshold, int min_len) {
    return guarded([&]() -> GDP_RETCODE {
        if (!ctx) { gdp::set_error("null context"); return GDP_ERROR; }
        return ctx->impl.set_model(model ? &model->impl : nullptr, threshold, min_len);
    });
}

GDP_RETCODE gdp_batch_set_model(gdp_batch *b, const gdp_mlp *model, float threshold, int min_len) {
    return guarded([&]() -> GDP_RETCODE {
        if (!b) { gdp::set_error("null batch"); return GDP_ERROR; }
        return b->impl.set_model(model ? &model->impl : nullptr, threshold, min_len);
    });
}

GDP_RETCODE gdp_context_trace(gdp_context *ctx, double *lbs, double *ubs, int capacity, float *features,
                              float *labels, int *n_samples, gdp_stats *stats) {
    return guarded([&]() -> GDP_RETCODE {
        if (!ctx || !lbs || !ubs) { gdp::set_error("null context or bounds"); return GDP_ERROR; }
        const auto t0 = std::chrono::steady_clock::now();
        const GDP_RETCODE rc = ctx->impl.trace(lbs, ubs, capacity, features, labels, n_samples, stats);
        if (stats)
            stats->total_ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    });
}

GDP_RETCODE gdp_autotune(int n_cons, int n_vars, int nnz, const int *col, const int *row_ptr, const double *val,
                         const double *lhs, const double *rhs, const double *lbs, const double *ubs,
                         const int *vartypes, const gdp_options *base, int repeats, gdp_options *best,
                         double *best_ms, gdp_tune_trial *trials, int max_trials, int *n_trials) {
    return guarded([&]() -> GDP_RETCODE {
        return gdp::autotune(n_cons, n_vars, nnz, col, row_ptr, val, lhs, rhs, lbs, ubs, vartypes, base, repeats,
                             best, best_ms, trials, max_trials, n_trials);
    });
}

GDP_RETCODE gdp_autotune_clear_cache(void) {
    return guarded([&]() -> GDP_RETCODE { return gdp::autotune_clear_cache(); });
}

namespace {
GDP_RETCODE timer_status(int e) {
    if (e == -1) {
        gdp::set_error("phase timers are compiled only into a library built with GDP_PHASE_TIMERS");
        return GDP_NOTIMPLEMENTED;
    }
    if (e != 0) {
        gdp::set_error(std::string("phase timers: ") + cudaGetErrorString((cudaError_t)e));
        return GDP_ERROR;
    }
    return GDP_OKAY;
}
}  // namespace

GDP_RETCODE gdp_phase_timers_clear(void) {
    return guarded([&]() -> GDP_RETCODE { return timer_status(gdp::phase_timers_clear()); });
}

GDP_RETCODE gdp_phase_timers_read(unsigned long long *wall, unsigned long long *busy, unsigned long long *pass,
                                  int rounds) {
    return guarded([&]() -> GDP_RETCODE { return timer_status(gdp::phase_timers_read(wall, busy, pass, rounds)); });
}

GDP_RETCODE gdp_context_destroy(gdp_context *ctx) {
    return guarded([&]() -> GDP_RETCODE {
        delete ctx;
        return GDP_OKAY;
    });
}

GDP_RETCODE gdp_propagate(gdp_context *ctx, double *lbs, double *ubs, gdp_stats *stats) {
    return guarded([&]() -> GDP_RETCODE {
        if (!ctx || !lbs || !ubs) { gdp::set_error("null argument"); return GDP_ERROR; }
        const auto t0 = std::chrono::steady_clock::now();
        if (stats) *stats = gdp_stats{};
        const GDP_RETCODE rc = ctx->impl.propagate_host(lbs, ubs, stats);
        if (stats)
            stats->total_ms =
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    });
}

GDP_RETCODE gdp_propagate_into(gdp_context *ctx, const double *lbs_in, const double *ubs_in, double *lbs_out,
                               double *ubs_out, gdp_stats *stats) {
    return guarded([&]() -> GDP_RETCODE {
        if (!ctx || !lbs_in || !ubs_in || !lbs_out || !ubs_out) {
            gdp::set_error("null argument");
            return GDP_ERROR;
        }
        const auto t0 = std::chrono::steady_clock::now();
        if (stats) *stats = gdp_stats{};
        const long long n = ctx->impl.n;
        // chunked copies on the host threads (one thread copies a few GB/s)
        const long long chunk = 1 << 16;
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (n + chunk - 1) / chunk; c++) {
            const long long b = c * chunk, len = std::min(chunk, n - b);
            if (lbs_out != lbs_in) std::memcpy(lbs_out + b, lbs_in + b, sizeof(double) * (size_t)len);
            if (ubs_out != ubs_in) std::memcpy(ubs_out + b, ubs_in + b, sizeof(double) * (size_t)len);
        }
        const GDP_RETCODE rc = ctx->impl.propagate_host(lbs_out, ubs_out, stats);
        if (stats)
            stats->total_ms =
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    });
}

GDP_RETCODE gdp_propagate_device(gdp_context *ctx, double *d_lbs, double *d_ubs, void *stream,
                                 gdp_stats *stats) {
    return guarded([&]() -> GDP_RETCODE {
        if (!ctx || !d_lbs || !d_ubs) { gdp::set_error("null argument"); return GDP_ERROR; }
        const auto t0 = std::chrono::steady_clock::now();
        if (stats) *stats = gdp_stats{};
        const GDP_RETCODE rc = ctx->impl.propagate_device(d_lbs, d_ubs, (cudaStream_t)stream, stats);
        if (stats)
            stats->total_ms =
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    });
}

GDP_RETCODE gdp_context_set_options(gdp_context *ctx, int max_rounds, int sync_type) {
    if (!ctx) { gdp::set_error("null context"); return GDP_ERROR; }
    if (sync_type < CPU_LOOP || sync_type > MEGAKERNEL) { gdp::set_error("Unknown sync type"); return GDP_ERROR; }
    ctx->impl.opts.max_rounds = max_rounds > 0 ? max_rounds : GDP_MAX_NUM_ROUNDS;
    ctx->impl.opts.sync_type = sync_type;
    ctx->impl.P.max_rounds = ctx->impl.opts.max_rounds;
    // the GPU_LOOP graph holds the round cap in its captured kernel arguments
    if (ctx->impl.graph_exec) { cudaGraphExecDestroy(ctx->impl.graph_exec); ctx->impl.graph_exec = nullptr; }
    if (ctx->impl.graph) { cudaGraphDestroy(ctx->impl.graph); ctx->impl.graph = nullptr; }
    return GDP_OKAY;
}

GDP_RETCODE gdp_context_layout(const gdp_context *ctx, long long out[6]) {
    if (!ctx || !out) { gdp::set_error("null argument"); return GDP_ERROR; }
    out[0] = ctx->impl.n_srows;
    out[1] = ctx->impl.n_slices;
    out[2] = ctx->impl.n_lrows;
    out[3] = ctx->impl.n_tiles;
    out[4] = ctx->impl.sell_elems;
    out[5] = ctx->impl.mega_grid;
    return GDP_OKAY;
}

GDP_RETCODE gdp_propagate_once(int n_cons, int n_vars, int nnz, const int *col, const int *row_ptr,
                               const double *val, const double *lhs, const double *rhs, double *lbs,
                               double *ubs, const int *vartypes, const gdp_options *opts,
                               gdp_stats *stats) {
    return guarded([&]() {
        return propagate_once_impl(n_cons, n_vars, nnz, col, row_ptr, val, lhs, rhs, lbs, ubs, vartypes,
                                   opts, stats);
    });
}

// ---- reference interface.h ------------------------------------------------
GDP_RETCODE propagateConstraintsGPUAtomicDouble(const int n_cons, const int n_vars, const int nnz,
                                                const int *csr_col_indices, const int *csr_row_ptrs,
                                                const double *csr_vals, const double *lhss,
                                                const double *rhss, double *lbs, double *ubs,
                                                const int *vartypes, const int sync_type) {
    return guarded([&]() -> GDP_RETCODE {
        if (sync_type < CPU_LOOP || sync_type > MEGAKERNEL) {
            gdp::set_error("Unknown sync type");
            return GDP_ERROR;
        }
        gdp_options o;
        gdp_default_options(&o);
        o.sync_type = sync_type;
        return propagate_once_impl(n_cons, n_vars, nnz, csr_col_indices, csr_row_ptrs, csr_vals, lhss,
                                   rhss, lbs, ubs, vartypes, &o, nullptr);
    });
}

GDP_RETCODE propagateConstraintsGPUReductionDouble(const int n_cons, const int n_vars, const int nnz,
                                                   const int *csr_col_indices, const int *csr_row_ptrs,
                                                   const double *csr_vals, const double *lhss,
                                                   const double *rhss, double *lbs, double *ubs,
                                                   const int *vartypes) {
    return guarded([&]() -> GDP_RETCODE {
        gdp_options o;
        gdp_default_options(&o);
        return propagate_once_impl(n_cons, n_vars, nnz, csr_col_indices, csr_row_ptrs, csr_vals, lhss,
                                   rhss, lbs, ubs, vartypes, &o, nullptr);
    });
}

static GDP_RETCODE not_implemented(const char *what) {
    gdp::set_error(std::string(what) + " is not implemented: this library is the FP64 GPU path only");
    return GDP_NOTIMPLEMENTED;
}

GDP_RETCODE propagateConstraintsGPUReductionFloat(const int, const int, const int, const int *, const int *,
                                                  const float *, const float *, const float *, float *,
                                                  float *, const int *) {
    return not_implemented("propagateConstraintsGPUReductionFloat");
}

GDP_RETCODE propagateConstraintsGPUAtomicFloat(const int, const int, const int, const int *, const int *,
                                               const float *, const float *, const float *, float *, float *,
                                               const int *, const int) {
    return not_implemented("propagateConstraintsGPUAtomicFloat");
}

GDP_RETCODE propagateConstraintsSequentialDouble(const int, const int, const int, const int *, const int *,
                                                 const double *, const double *, const double *, double *,
                                                 double *, const int *) {
    return not_implemented("propagateConstraintsSequentialDouble");
}

GDP_RETCODE propagateConstraintsSequentialFloat(const int, const int, const int, const int *, const int *,
                                                const float *, const float *, const float *, float *,
                                                float *, const int *) {
    return not_implemented("propagateConstraintsSequentialFloat");
}

GDP_RETCODE propagateConstraintsFullOMPDouble(const int, const int, const int, const int *, const int *,
                                              const double *, const double *, const double *, double *,
                                              double *, const int *) {
    return not_implemented("propagateConstraintsFullOMPDouble");
}

GDP_RETCODE propagateConstraintsFullOMPFloat(const int, const int, const int, const int *, const int *,
                                             const float *, const float *, const float *, float *, float *,
                                             const int *) {
    return not_implemented("propagateConstraintsFullOMPFloat");
}

GDP_RETCODE propagateConstraintsSequentialDisjointDouble(const int, const int, const int, const int *,
                                                         const int *, const double *, const double *,
                                                         const double *, double *, double *, const int *) {
    return not_implemented("propagateConstraintsSequentialDisjointDouble");
}

GDP_RETCODE sequentialPropagateWithMeasureDouble(const int, const int, const int, const int *, const int *,
                                                 const double *, const double *, const double *, double *,
                                                 double *, const int *) {
    return not_implemented("sequentialPropagateWithMeasureDouble");
}

GDP_RETCODE atomicPropagateWithMeasureDouble(const int, const int, const int, const int *, const int *,
                                             const double *, const double *, const double *, double *,
                                             double *, const int *) {
    return not_implemented("atomicPropagateWithMeasureDouble");
}

}  // extern "C"
#pragma GCC visibility pop

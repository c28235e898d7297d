// gdp_batch_host.cu -- host side of the batched engine: builds the units
// (per-instance layouts, or per-node state over one shared layout), the batch
// queues, and runs a batch as one captured CUDA graph.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <numeric>
#include <string>

#include "gdp_batch.h"

namespace gdp {

#define GDP_BCUDA(call)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call);      \
            return GDP_ERROR;                                                                    \
        }                                                                                        \
    } while (0)

Batch::~Batch() {
    if (stream_) cudaStreamSynchronize(stream_);
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (h_lb_) cudaFreeHost(h_lb_);
    if (h_ub_) cudaFreeHost(h_ub_);
    if (h_flags_) cudaFreeHost(h_flags_);
    if (h_flags_init_) cudaFreeHost(h_flags_init_);
    if (h_rounds_) cudaFreeHost(h_rounds_);
    if (h_seed_) cudaFreeHost(h_seed_);
    if (stream_) cudaStreamDestroy(stream_);
}

GDP_RETCODE Batch::init_instances(int n_inst, const int *n_cons, const int *n_vars, const int *nnz,
                                  const int *const *col, const int *const *row_ptr, const double *const *val,
                                  const double *const *lhs, const double *const *rhs,
                                  const int *const *vartype, const gdp_options *o) {
    if (n_inst <= 0 || n_inst > 65535) {
        set_error("a batch holds 1 to 65535 instances");
        return GDP_ERROR;
    }
    gdp_options opts;
    gdp_default_options(&opts);
    if (o) opts = *o;
    // units in heaviest-first order, so that full sweeps start with the big items
    member_of_unit_.resize(n_inst);
    std::iota(member_of_unit_.begin(), member_of_unit_.end(), 0);
    std::stable_sort(member_of_unit_.begin(), member_of_unit_.end(),
                     [&](int a, int b) { return nnz[a] > nnz[b]; });
    inst_.resize(n_inst);
    for (int u = 0; u < n_inst; u++) {
        const int k = member_of_unit_[u];
        inst_[u].reset(new Context());
        if (inst_[u]->init(n_cons[k], n_vars[k], nnz[k], col[k], row_ptr[k], val[k], lhs[k], rhs[k], vartype[k],
                           &opts) != GDP_OKAY) {
            set_error("instance " + std::to_string(k) + ": " + last_error());
            return GDP_ERROR;
        }
    }
    n_units = n_inst;
    nodes = false;
    max_rounds = inst_[0]->opts.max_rounds;
    units_h_.resize(n_units);
    for (int u = 0; u < n_units; u++) {
        units_h_[u] = inst_[u]->P;
        units_h_[u].defer_exact = 0;  // the batch loop runs exact passes in place
    }
    // per-unit batch state: slice stamps
    for (int u = 0; u < n_units; u++) {
        DevProblem &Q = units_h_[u];
        Q.slice_stamp = (int *)arena_.alloc_bytes(sizeof(int) * (size_t)std::max(Q.n_slices, 1));
        if (!Q.slice_stamp) { set_error("device allocation failed (slice stamps)"); return GDP_ERROR; }
    }
    seed_mode_.assign(n_units, 0);
    ref_ = nullptr;
    return finish_init(opts.device, opts.ctas_per_sm);
}

GDP_RETCODE Batch::init_nodes(Context *ctx, int n_nodes) {
    if (!ctx || n_nodes <= 0 || n_nodes > 65535) {
        set_error("a node batch needs a context and 1 to 65535 nodes");
        return GDP_ERROR;
    }
    base_ = ctx;
    n_units = n_nodes;
    nodes = true;
    max_rounds = ctx->opts.max_rounds;
    member_of_unit_.resize(n_nodes);
    std::iota(member_of_unit_.begin(), member_of_unit_.end(), 0);
    const DevProblem &S = ctx->P;
    const int n = std::max(S.n, 1), npos = std::max(S.n_srows + S.n_lrows, 1);
    units_h_.assign(n_units, S);
    for (int u = 0; u < n_units; u++) units_h_[u].defer_exact = 0;  // exact passes run in place
    for (int u = 0; u < n_units; u++) {
        DevProblem &Q = units_h_[u];
        Q.bnd = (double2 *)arena_.alloc_bytes(sizeof(double2) * (size_t)n);
        Q.bnd_nxt = (double2 *)arena_.alloc_bytes(sizeof(double2) * (size_t)n);
        Q.bnd32 = (float2 *)arena_.alloc_bytes(sizeof(float2) * (size_t)n);  // 8-byte copies
        Q.chg = (unsigned *)arena_.alloc_bytes(sizeof(unsigned) * (size_t)std::max(S.n_chg_words, 1));
        Q.mark = (int *)arena_.alloc_bytes(sizeof(int) * (size_t)npos);
        Q.slice_stamp = (int *)arena_.alloc_bytes(sizeof(int) * (size_t)std::max(S.n_slices, 1));
        Q.tile_part = (TilePart *)arena_.alloc_bytes(sizeof(TilePart) * (size_t)std::max(S.n_tiles, 1));
        Q.tile_scr = (TileScr *)arena_.alloc_bytes(sizeof(TileScr) * (size_t)std::max(S.n_tiles, 1));
        Q.row_exact = (int *)arena_.alloc_bytes(sizeof(int) * (size_t)std::max(S.n_lrows, 1));
        if (!Q.bnd || !Q.bnd_nxt || !Q.bnd32 || !Q.chg || !Q.mark || !Q.slice_stamp || !Q.tile_part || !Q.tile_scr ||
            !Q.row_exact) {
            set_error("device allocation failed (node state)");
            return GDP_ERROR;
        }
    }
    seed_mode_.assign(n_units, 1);
    ref_ = ctx->P.bnd;  // read only while the context's last propagation is certified
    return finish_init(ctx->opts.device, ctx->opts.ctas_per_sm);
}

GDP_RETCODE Batch::finish_init(int device, int ctas_per_sm) {
    GDP_BCUDA(cudaSetDevice(device));
    GDP_BCUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    GDP_BCUDA(cudaEventCreate(&ev0_));
    GDP_BCUDA(cudaEventCreate(&ev1_));
    // variables of every unit, back to back in the staging buffers
    var_base_.assign(n_units + 1, 0);
    std::vector<int> wbase(n_units + 1, 0);
    long long cap_entries = 0, cap_tiles = 0;
    max_unit_n_ = 0;
    for (int u = 0; u < n_units; u++) {
        const DevProblem &Q = units_h_[u];
        var_base_[u + 1] = var_base_[u] + Q.n;
        wbase[u + 1] = wbase[u] + Q.n_chg_words;
        cap_entries += (long long)Q.n_slices + Q.n_tiles;
        cap_tiles += Q.n_mtiles;
        max_unit_n_ = std::max(max_unit_n_, std::max(Q.n, Q.n_srows + Q.n_lrows));
        if (!Q.var_ptr) {
            set_error("unit without a marking index");
            return GDP_ERROR;
        }
    }
    total_vars_ = var_base_[n_units];
    if (cap_entries >= (long long)UINT_MAX || cap_tiles >= (long long)UINT_MAX || wbase[n_units] < 0) {
        set_error("batch too large for 32-bit work queues");
        return GDP_ERROR;
    }
    // shared round flags: one contiguous array, so one copy returns every unit's result
    d_flags_ = (RoundFlags *)arena_.alloc_bytes(sizeof(RoundFlags) * 3 * (size_t)n_units);
    if (!d_flags_) { set_error("device allocation failed (flags)"); return GDP_ERROR; }
    for (int u = 0; u < n_units; u++) units_h_[u].flags = d_flags_ + 3 * u;
    GDP_BCUDA(cudaMallocHost(&h_flags_, sizeof(RoundFlags) * 3 * (size_t)n_units));
    GDP_BCUDA(cudaMallocHost(&h_flags_init_, sizeof(RoundFlags) * 3 * (size_t)n_units));
    std::memset(h_flags_init_, 0, sizeof(RoundFlags) * 3 * (size_t)n_units);
    for (int u = 0; u < n_units; u++) {
        h_flags_init_[3 * u].infeasible_var = INT_MAX;
        h_flags_init_[3 * u].infeasible_row = INT_MAX;
    }
    GDP_BCUDA(cudaMallocHost(&h_rounds_, sizeof(int) * 2));
    GDP_BCUDA(cudaMallocHost(&h_seed_, sizeof(int) * (size_t)n_units));
    GDP_BCUDA(cudaMallocHost(&h_lb_, sizeof(double) * (size_t)std::max<long long>(total_vars_, 1)));
    GDP_BCUDA(cudaMallocHost(&h_ub_, sizeof(double) * (size_t)std::max<long long>(total_vars_, 1)));

    auto dev = [&](size_t bytes) { return arena_.alloc_bytes(std::max<size_t>(bytes, 16)); };
    std::memset(&B_, 0, sizeof(B_));
    B_.n_units = n_units;
    B_.units = (DevProblem *)dev(sizeof(DevProblem) * (size_t)n_units);
    B_.wbase = (const int *)dev(sizeof(int) * (size_t)(n_units + 1));
    B_.total_words = wbase[n_units];
    B_.max_rounds = max_rounds;
    B_.spin_limit = units_h_[0].spin_limit;
    B_.cap_entries = (unsigned)std::max<long long>(cap_entries, 1);
    B_.entries = (unsigned long long *)dev(sizeof(unsigned long long) * 2 * (size_t)B_.cap_entries);
    B_.cap_tiles = (unsigned)std::max<long long>(cap_tiles, 1);
    B_.cq = (unsigned long long *)dev(sizeof(unsigned long long) * (size_t)B_.cap_tiles);
    B_.xq = (unsigned long long *)dev(sizeof(unsigned long long) * (size_t)B_.cap_tiles);
    B_.ctr = (unsigned *)dev(sizeof(unsigned) * 8);
    B_.tail = (unsigned *)dev(sizeof(unsigned) * 4);
    B_.fs_unit = (int *)dev(sizeof(int) * (size_t)n_units);
    B_.fs_prefix = (int *)dev(sizeof(int) * (size_t)(n_units + 1));
    B_.n_fs = (int *)dev(sizeof(int));
    B_.barrier = (unsigned *)dev(sizeof(unsigned) * 2);
    // error and rounds_out adjacent: one copy reads both
    int *misc = (int *)dev(sizeof(int) * 3);
    B_.error = misc;
    B_.rounds_out = misc + 1;
    B_.n_pending = misc + 2;
    d_lb_ = (double *)dev(sizeof(double) * (size_t)total_vars_);
    d_ub_ = (double *)dev(sizeof(double) * (size_t)total_vars_);
    d_var_base_ = (long long *)dev(sizeof(long long) * (size_t)(n_units + 1));
    d_seed_mode_ = (int *)dev(sizeof(int) * (size_t)n_units);
    if (!B_.units || !B_.wbase || !B_.entries || !B_.cq || !B_.xq || !B_.ctr || !B_.tail || !B_.fs_unit ||
        !B_.fs_prefix || !B_.n_fs || !B_.barrier || !misc || !d_lb_ || !d_ub_ || !d_var_base_ || !d_seed_mode_) {
        set_error("device allocation failed (batch)");
        return GDP_ERROR;
    }
    GDP_BCUDA(cudaMemcpyAsync(B_.units, units_h_.data(), sizeof(DevProblem) * (size_t)n_units,
                              cudaMemcpyHostToDevice, stream_));
    GDP_BCUDA(cudaMemcpyAsync((void *)B_.wbase, wbase.data(), sizeof(int) * (size_t)(n_units + 1),
                              cudaMemcpyHostToDevice, stream_));
    GDP_BCUDA(cudaMemcpyAsync(d_var_base_, var_base_.data(), sizeof(long long) * (size_t)(n_units + 1),
                              cudaMemcpyHostToDevice, stream_));
    device_ = device;
    ctas_per_sm_ = ctas_per_sm;
    if (size_grid() != GDP_OKAY) return GDP_ERROR;
    GDP_BCUDA(cudaStreamSynchronize(stream_));
    return GDP_OKAY;
}

// Cooperative grid of the batch loop instantiation in use.
GDP_RETCODE Batch::size_grid() {
    int bps = 0, sms = 0;
    GDP_BCUDA((cudaError_t)batch_occupancy(&bps, learned_));
    GDP_BCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    if (ctas_per_sm_ > 0) bps = std::min(bps, ctas_per_sm_);
    grid = std::max(1, bps) * sms;
    return GDP_OKAY;
}

GDP_RETCODE Batch::set_model(const Mlp *m, float threshold, int min_len) {
    if (nodes) {
        set_error("learned marking in a batch needs instance members");
        return GDP_ERROR;
    }
    GDP_BCUDA(cudaStreamSynchronize(stream_));
    for (int u = 0; u < n_units; u++) {
        if (inst_[u]->set_model(m, threshold, min_len) != GDP_OKAY) return GDP_ERROR;
        const DevProblem &S = inst_[u]->P;
        DevProblem &Q = units_h_[u];
        Q.learned = S.learned;
        Q.tau = S.tau;
        Q.learn_min_len = S.learn_min_len;
        Q.mlp = S.mlp;
        Q.dirty = S.dirty;
        Q.dcount = S.dcount;
        Q.last_proc = S.last_proc;
        Q.last_tight = S.last_tight;
        Q.rstat = S.rstat;
        Q.rinfo = S.rinfo;
        Q.trace_n = S.trace_n;
    }
    learned_ = m != nullptr;
    GDP_BCUDA(cudaMemcpyAsync(B_.units, units_h_.data(), sizeof(DevProblem) * (size_t)n_units,
                              cudaMemcpyHostToDevice, stream_));
    GDP_BCUDA(cudaStreamSynchronize(stream_));
    if (size_grid() != GDP_OKAY) return GDP_ERROR;
    // the captured graph holds the other loop instantiation and grid: capture again
    if (graph_exec_) { cudaGraphExecDestroy(graph_exec_); graph_exec_ = nullptr; }
    if (graph_) { cudaGraphDestroy(graph_); graph_ = nullptr; }
    graph_failed_ = false;
    return GDP_OKAY;
}

// Member bounds to and from the pinned staging arrays, in pieces of 64K
// variables spread over the host threads: one thread copies a few GB/s, and
// node batches move hundreds of MB each way.
namespace {
template <class F>
void for_each_piece(int n_units, const std::vector<long long> &var_base, F &&f) {
    constexpr long long kPiece = 1 << 16;
    std::vector<long long> first(n_units + 1, 0);  // first piece of each unit
    for (int u = 0; u < n_units; u++)
        first[u + 1] = first[u] + (var_base[u + 1] - var_base[u] + kPiece - 1) / kPiece;
    const long long n_pieces = first[n_units];
#pragma omp parallel for schedule(dynamic, 4)
    for (long long q = 0; q < n_pieces; q++) {
        // the unit whose pieces include q (units without variables have none)
        const int u = (int)(std::upper_bound(first.begin(), first.end(), q) - first.begin()) - 1;
        const long long off = (q - first[u]) * kPiece;
        f(u, off, (size_t)std::min(kPiece, var_base[u + 1] - var_base[u] - off));
    }
}
}  // namespace

void Batch::copy_in(const double *const *lbs, const double *const *ubs) {
    for_each_piece(n_units, var_base_, [&](int u, long long off, size_t n) {
        const int k = member_of_unit_[u];
        std::memcpy(h_lb_ + var_base_[u] + off, lbs[k] + off, sizeof(double) * n);
        std::memcpy(h_ub_ + var_base_[u] + off, ubs[k] + off, sizeof(double) * n);
    });
}

void Batch::copy_out(double *const *lbs, double *const *ubs) {
    for_each_piece(n_units, var_base_, [&](int u, long long off, size_t n) {
        const int k = member_of_unit_[u];
        std::memcpy(lbs[k] + off, h_lb_ + var_base_[u] + off, sizeof(double) * n);
        std::memcpy(ubs[k] + off, h_ub_ + var_base_[u] + off, sizeof(double) * n);
    });
}

// The device part of one batch call, in stream order.
GDP_RETCODE Batch::enqueue(cudaStream_t s) {
    const size_t vbytes = sizeof(double) * (size_t)total_vars_;
    if (vbytes) {
        GDP_BCUDA(cudaMemcpyAsync(d_lb_, h_lb_, vbytes, cudaMemcpyHostToDevice, s));
        GDP_BCUDA(cudaMemcpyAsync(d_ub_, h_ub_, vbytes, cudaMemcpyHostToDevice, s));
    }
    GDP_BCUDA(cudaMemcpyAsync(d_seed_mode_, h_seed_, sizeof(int) * (size_t)n_units, cudaMemcpyHostToDevice, s));
    GDP_BCUDA(cudaMemcpyAsync(d_flags_, h_flags_init_, sizeof(RoundFlags) * 3 * (size_t)n_units,
                              cudaMemcpyHostToDevice, s));
    GDP_BCUDA(cudaMemsetAsync(B_.ctr, 0, sizeof(unsigned) * 8, s));
    GDP_BCUDA(cudaMemsetAsync(B_.tail, 0, sizeof(unsigned) * 4, s));
    GDP_BCUDA(cudaMemsetAsync(B_.barrier, 0, sizeof(unsigned) * 2, s));
    GDP_BCUDA(cudaMemsetAsync(B_.error, 0, sizeof(int) * 3, s));
    // external records: inside a stream capture they become graph event nodes
    GDP_BCUDA(cudaEventRecordWithFlags(ev0_, s, cudaEventRecordExternal));
    GDP_BCUDA((cudaError_t)launch_batch(B_, grid, d_lb_, d_ub_, d_lb_, d_ub_, d_var_base_, max_unit_n_, ref_,
                                        d_seed_mode_, learned_, s));
    GDP_BCUDA(cudaEventRecordWithFlags(ev1_, s, cudaEventRecordExternal));
    if (vbytes) {
        GDP_BCUDA(cudaMemcpyAsync(h_lb_, d_lb_, vbytes, cudaMemcpyDeviceToHost, s));
        GDP_BCUDA(cudaMemcpyAsync(h_ub_, d_ub_, vbytes, cudaMemcpyDeviceToHost, s));
    }
    GDP_BCUDA(cudaMemcpyAsync(h_flags_, d_flags_, sizeof(RoundFlags) * 3 * (size_t)n_units,
                              cudaMemcpyDeviceToHost, s));
    GDP_BCUDA(cudaMemcpyAsync(h_rounds_, B_.error, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
    return GDP_OKAY;
}

GDP_RETCODE Batch::propagate(const double *const *lbs_in, const double *const *ubs_in, double *const *lbs_out,
                             double *const *ubs_out, gdp_stats *member_stats, gdp_stats *total) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!lbs_in || !ubs_in || !lbs_out || !ubs_out) {
        set_error("null bound arrays");
        return GDP_ERROR;
    }
    for (int u = 0; u < n_units; u++) {
        const int k = member_of_unit_[u];
        if (var_base_[u + 1] > var_base_[u] && (!lbs_in[k] || !ubs_in[k] || !lbs_out[k] || !ubs_out[k])) {
            set_error("null bounds for member " + std::to_string(k));
            return GDP_ERROR;
        }
    }
    copy_in(lbs_in, ubs_in);
    // nodes start from the marks of their differences to the context's
    // fixpoint when its last propagation certified one; otherwise they sweep
    const int seed = nodes && base_ && base_->certified ? 1 : 0;
    for (int u = 0; u < n_units; u++) h_seed_[u] = nodes ? seed : seed_mode_[u];
    if (use_graph && !graph_exec_ && !graph_failed_) {
        cudaGraph_t g = nullptr;
        bool ok = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        const bool enq = ok && enqueue(stream_) == GDP_OKAY;
        const cudaError_t ec = cudaStreamEndCapture(stream_, &g);
        ok = ok && enq && ec == cudaSuccess && g;
        cudaGraphExec_t ge = nullptr;
        if (ok) ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
        if (ok) {
            graph_ = g;
            graph_exec_ = ge;
        } else {
            if (g) cudaGraphDestroy(g);
            graph_failed_ = true;  // launch the same sequence directly from now on
        }
        cudaGetLastError();
    }
    graph_ok = graph_exec_ != nullptr;
    if (graph_ok) {
        GDP_BCUDA(cudaGraphLaunch(graph_exec_, stream_));
    } else if (enqueue(stream_) != GDP_OKAY) {
        return GDP_ERROR;
    }
    GDP_BCUDA(cudaStreamSynchronize(stream_));
    if (h_rounds_[0] != kErrNone) {
        set_error("batch device error " + std::to_string(h_rounds_[0]) +
                  (h_rounds_[0] == kErrBarrierTimeout ? " (grid barrier wait exceeded its limit)"
                                                      : " (work queue overflow)"));
        if (total) total->device_error = h_rounds_[0];
        return GDP_ERROR;
    }
    copy_out(lbs_out, ubs_out);
    float ms = -1.f;
    if (cudaEventElapsedTime(&ms, ev0_, ev1_) != cudaSuccess) {
        ms = -1.f;
        cudaGetLastError();  // leave no error behind for the caller's next check
    }
    const double total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    gdp_stats tot{};
    tot.converged = 1;
    tot.infeasible_var = -1;
    tot.infeasible_row = -1;
    for (int u = 0; u < n_units; u++) {
        const RoundFlags &f = h_flags_[3 * u];
        gdp_stats st{};
        st.rounds = f.rounds;
        st.infeasible = f.infeasible;
        st.infeasible_var = (f.infeasible && f.infeasible_var != INT_MAX) ? f.infeasible_var : -1;
        st.infeasible_row = (f.infeasible && f.infeasible_row != INT_MAX) ? f.infeasible_row : -1;
        st.converged = (f.infeasible || !f.change) ? 1 : 0;
        st.kernel_launches = 5;
        st.changed_vars = (long long)f.changed_vars;
        st.rows_processed = (long long)f.rows_proc;
        st.nnz_processed = (long long)f.nnz_proc;
        st.nnz_exact = (long long)f.nnz_exact;
        st.rows_deferred = (long long)f.rows_deferred;
        st.divisions = (long long)f.divisions;
        st.rows_exact = (long long)f.rows_exact;
        st.rows_go = (long long)f.rows_go;
        st.rows_seqmax = (long long)f.rows_seqmax;
        st.rows_drift = (long long)f.rows_drift;
        st.nnz_drift = (long long)f.nnz_drift;
        st.full_rounds = f.full_rounds;
        st.bytes_algorithmic = 12.0 * (double)f.nnz_proc + 20.0 * (double)f.rows_proc +
                               36.0 * (double)(var_base_[u + 1] - var_base_[u]) * (double)f.rounds;
        st.device_ms = ms;
        st.total_ms = total_ms;
        if (member_stats) member_stats[member_of_unit_[u]] = st;
        tot.rounds = std::max(tot.rounds, st.rounds);
        tot.converged &= st.converged;
        tot.infeasible += st.infeasible;
        tot.changed_vars += st.changed_vars;
        tot.rows_processed += st.rows_processed;
        tot.nnz_processed += st.nnz_processed;
        tot.nnz_exact += st.nnz_exact;
        tot.rows_deferred += st.rows_deferred;
        tot.divisions += st.divisions;
        tot.rows_exact += st.rows_exact;
        tot.rows_go += st.rows_go;
        tot.rows_seqmax += st.rows_seqmax;
        tot.rows_drift += st.rows_drift;
        tot.nnz_drift += st.nnz_drift;
        tot.full_rounds = std::max(tot.full_rounds, st.full_rounds);
        tot.bytes_algorithmic += st.bytes_algorithmic;
    }
    tot.kernel_launches = 5;
    tot.device_ms = ms;
    tot.total_ms = total_ms;
    if (total) *total = tot;
    return GDP_OKAY;
}

}  // namespace gdp

// gdp_context.cu -- host side of the propagator: input validation, device
// layout (SELL slices of thread rows, tiles of split rows), device buffers and
// the round-loop drivers.
//
// Replaces the reference's per-call host driver propagateConstraintsGPUAtomic
// (src/propagators/GPU_propagator.cuh:98-268): uploads, row binning
// (fill_row_blocks, src/kernels/util_kernels.cu:12-62) and the three round
// loops. CUDA errors return GDP_ERROR with a message instead of exit()
// (reference src/cuda_def.cuh:10-15).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gdp_context.h"

namespace gdp {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }
const char *last_error() { return g_last_error.c_str(); }

#define GDP_CUDA(expr)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (cudaError_t)(expr);                                           \
        if (e_ != cudaSuccess) {                                                        \
            set_error(std::string(#expr) + " failed: " + cudaGetErrorString(e_));       \
            return GDP_ERROR;                                                           \
        }                                                                               \
    } while (0)

// ---------------------------------------------------------------------------
Arena::~Arena() {
    for (void *p : ptrs) cudaFree(p);
}

void *Arena::alloc_bytes(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    ptrs.push_back(p);
    return p;
}

// ---------------------------------------------------------------------------
GDP_RETCODE validate_csr(int m, int n, int nnz, const int *col, const int *row_ptr,
                         const double *val, const int *vartype) {
    if (m < 0 || n < 0 || nnz < 0) { set_error("negative problem size"); return GDP_ERROR; }
    if (!col || !row_ptr || !val || !vartype) { set_error("null input array"); return GDP_ERROR; }
    if (row_ptr[0] != 0 || row_ptr[m] != nnz) {
        set_error("csr_row_ptrs must start at 0 and end at nnz");
        return GDP_ERROR;
    }
    for (int i = 0; i < m; i++)
        if (row_ptr[i + 1] < row_ptr[i]) { set_error("csr_row_ptrs is not monotone"); return GDP_ERROR; }
    for (int k = 0; k < nnz; k++)
        if ((unsigned)col[k] >= (unsigned)n) {
            set_error("column index out of range at non-zero " + std::to_string(k));
            return GDP_ERROR;
        }
    for (int k = 0; k < nnz; k++)
        if (!std::isfinite(val[k])) {
            set_error("non-finite coefficient at non-zero " + std::to_string(k));
            return GDP_ERROR;
        }
    for (int j = 0; j < n; j++)
        if (vartype[j] != 0 && vartype[j] != 1 && vartype[j] != 3) {
            set_error("vartype must be 0, 1 or 3 (variable " + std::to_string(j) + ")");
            return GDP_ERROR;
        }
    return GDP_OKAY;
}

// ---------------------------------------------------------------------------
GDP_RETCODE Context::init(int m_, int n_, int nnz_, const int *col, const int *row_ptr,
                          const double *val, const double *lhs, const double *rhs,
                          const int *vartype, const gdp_options *o) {
    m = m_; n = n_; nnz = nnz_;
    gdp_default_options(&opts);
    if (o) opts = *o;
    if (opts.max_rounds <= 0) opts.max_rounds = GDP_MAX_NUM_ROUNDS;
    if (opts.thread_row_max <= 0) opts.thread_row_max = 1024;
    if (opts.split_tile <= 0) opts.split_tile = 4096;
    if (opts.sync_type < CPU_LOOP || opts.sync_type > MEGAKERNEL) {
        set_error("Unknown sync type");
        return GDP_ERROR;
    }
    if (!lhs || !rhs) { set_error("null lhs/rhs"); return GDP_ERROR; }
    if (validate_csr(m, n, nnz, col, row_ptr, val, vartype) != GDP_OKAY) return GDP_ERROR;

    GDP_CUDA(cudaSetDevice(opts.device));
    GDP_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    GDP_CUDA(cudaEventCreate(&ev0));
    GDP_CUDA(cudaEventCreate(&ev1));
    GDP_CUDA(cudaMallocHost(&h_flags, sizeof(RoundFlags) * 3));
    int sms = 0;
    GDP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opts.device));
    n_sms = sms;

    // ---- row binning (host) ----
    const int Lt = opts.thread_row_max;
    std::vector<int> len(m);
    int max_len = 0;
    for (int i = 0; i < m; i++) {
        len[i] = row_ptr[i + 1] - row_ptr[i];
        max_len = std::max(max_len, len[i]);
    }
    // counting sort of thread rows by length, longest first, stable by row index
    std::vector<int> cnt(Lt + 2, 0);
    std::vector<int> split_rows;
    for (int i = 0; i < m; i++) {
        if (len[i] == 0) continue;
        if (len[i] <= Lt) cnt[len[i]]++;
        else split_rows.push_back(i);
    }
    std::vector<int> start(Lt + 2, 0);
    int acc = 0;
    for (int L = Lt; L >= 1; L--) { start[L] = acc; acc += cnt[L]; }
    const int ns = acc;
    std::vector<int> order(ns);
    for (int i = 0; i < m; i++)
        if (len[i] >= 1 && len[i] <= Lt) order[start[len[i]]++] = i;
    std::stable_sort(split_rows.begin(), split_rows.end(),
                     [&](int a, int b) { return len[a] > len[b]; });

    n_srows = ns;
    n_slices = (ns + 31) / 32;
    std::vector<long long> slice_ptr(n_slices + 1, 0);
    for (int s = 0; s < n_slices; s++) slice_ptr[s + 1] = slice_ptr[s] + 32LL * len[order[32 * s]];
    sell_elems = slice_ptr[n_slices];
    std::vector<int> sell_col((size_t)std::max<long long>(sell_elems, 1), 0);
    std::vector<double> sell_val((size_t)std::max<long long>(sell_elems, 1), 0.0);
    std::vector<int> srow_len(std::max(ns, 1));
    std::vector<double> srow_lhs(std::max(ns, 1)), srow_rhs(std::max(ns, 1));
#pragma omp parallel for schedule(static)
    for (int s = 0; s < n_slices; s++) {
        for (int l = 0; l < 32; l++) {
            const int r = 32 * s + l;
            if (r >= ns) break;
            const int i = order[r];
            srow_len[r] = len[i];
            srow_lhs[r] = lhs[i];
            srow_rhs[r] = rhs[i];
            for (int k = 0; k < len[i]; k++) {
                const long long e = slice_ptr[s] + 32LL * k + l;
                sell_col[e] = col[row_ptr[i] + k];
                sell_val[e] = val[row_ptr[i] + k];
            }
        }
    }
    // split rows: CSR-contiguous, tiles of split_tile non-zeros
    n_lrows = (int)split_rows.size();
    std::vector<int> lrow_ptr(n_lrows + 1, 0), lrow_tile0(n_lrows + 1, 0);
    std::vector<double> lrow_lhs(std::max(n_lrows, 1)), lrow_rhs(std::max(n_lrows, 1));
    std::vector<int> tile_row, tile_begin, tile_end;
    for (int r = 0; r < n_lrows; r++) {
        const int i = split_rows[r];
        lrow_ptr[r + 1] = lrow_ptr[r] + len[i];
        lrow_lhs[r] = lhs[i];
        lrow_rhs[r] = rhs[i];
        lrow_tile0[r] = (int)tile_row.size();
        for (int b = lrow_ptr[r]; b < lrow_ptr[r + 1]; b += opts.split_tile) {
            tile_row.push_back(r);
            tile_begin.push_back(b);
            tile_end.push_back(std::min(b + opts.split_tile, lrow_ptr[r + 1]));
        }
    }
    lrow_tile0[n_lrows] = (int)tile_row.size();
    n_tiles = (int)tile_row.size();
    const long long lnnz = lrow_ptr[n_lrows];
    std::vector<int> lcol((size_t)std::max<long long>(lnnz, 1));
    std::vector<double> lval((size_t)std::max<long long>(lnnz, 1));
#pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < n_lrows; r++) {
        const int i = split_rows[r];
        std::memcpy(&lcol[lrow_ptr[r]], &col[row_ptr[i]], sizeof(int) * (size_t)len[i]);
        std::memcpy(&lval[lrow_ptr[r]], &val[row_ptr[i]], sizeof(double) * (size_t)len[i]);
    }
    rows_nonempty = (long long)ns + n_lrows;
    nnz_rows = nnz;

    // ---- upload ----
    auto up = [&](const void *src, size_t bytes) -> void * {
        void *d = arena.alloc_bytes(bytes);
        if (!d) return nullptr;
        if (bytes && cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, stream) != cudaSuccess)
            return nullptr;
        return d;
    };
#define GDP_UP(dst, T, vec, cnt_)                                                        \
    do {                                                                               \
        dst = (T *)up((vec).data(), sizeof(T) * (size_t)(cnt_));                       \
        if (!dst) { set_error("device allocation/upload failed for " #vec); return GDP_ERROR; } \
    } while (0)
    const long long *d_slice_ptr; const int *d_sell_col; const double *d_sell_val;
    const int *d_srow_len; const double *d_srow_lhs, *d_srow_rhs;
    GDP_UP(d_slice_ptr, const long long, slice_ptr, n_slices + 1);
    GDP_UP(d_sell_col, const int, sell_col, sell_col.size());
    GDP_UP(d_sell_val, const double, sell_val, sell_val.size());
    GDP_UP(d_srow_len, const int, srow_len, srow_len.size());
    GDP_UP(d_srow_lhs, const double, srow_lhs, srow_lhs.size());
    GDP_UP(d_srow_rhs, const double, srow_rhs, srow_rhs.size());
    const int *d_lcol, *d_lrow_tile0, *d_tile_row, *d_tile_begin, *d_tile_end;
    const double *d_lval, *d_lrow_lhs, *d_lrow_rhs;
    GDP_UP(d_lcol, const int, lcol, lcol.size());
    GDP_UP(d_lval, const double, lval, lval.size());
    GDP_UP(d_lrow_lhs, const double, lrow_lhs, lrow_lhs.size());
    GDP_UP(d_lrow_rhs, const double, lrow_rhs, lrow_rhs.size());
    GDP_UP(d_lrow_tile0, const int, lrow_tile0, lrow_tile0.size());
    if (tile_row.empty()) { tile_row.push_back(0); tile_begin.push_back(0); tile_end.push_back(0); }
    GDP_UP(d_tile_row, const int, tile_row, tile_row.size());
    GDP_UP(d_tile_begin, const int, tile_begin, tile_begin.size());
    GDP_UP(d_tile_end, const int, tile_end, tile_end.size());
    std::vector<unsigned char> is_cont(std::max(n, 1), 0);
    for (int j = 0; j < n; j++) is_cont[j] = vartype[j] == GDP_CONTINUOUS ? 1 : 0;
    const unsigned char *d_is_cont;
    GDP_UP(d_is_cont, const unsigned char, is_cont, is_cont.size());
#undef GDP_UP

    RowActsPOD *d_tile_part = (RowActsPOD *)arena.alloc_bytes(sizeof(RowActsPOD) * (size_t)std::max(n_tiles, 1));
    d_lb = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n, 1));
    d_ub = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n, 1));
    d_lb_nxt = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n, 1));
    d_ub_nxt = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n, 1));
    const int n_words = (n + 31) / 32;
    unsigned *d_chg = (unsigned *)arena.alloc_bytes(sizeof(unsigned) * (size_t)std::max(n_words, 1));
    d_flags = (RoundFlags *)arena.alloc_bytes(sizeof(RoundFlags) * 3);
    d_barrier = (unsigned *)arena.alloc_bytes(sizeof(unsigned) * 2);
    if (!d_tile_part || !d_lb || !d_ub || !d_lb_nxt || !d_ub_nxt || !d_chg || !d_flags || !d_barrier) {
        set_error("device allocation failed");
        return GDP_ERROR;
    }
    GDP_CUDA(cudaMemsetAsync(d_chg, 0, sizeof(unsigned) * (size_t)std::max(n_words, 1), stream));

    std::memset(&P, 0, sizeof(P));
    P.n = n;
    P.n_srows = n_srows; P.n_slices = n_slices;
    P.slice_ptr = d_slice_ptr; P.sell_col = d_sell_col; P.sell_val = d_sell_val;
    P.srow_len = d_srow_len; P.srow_lhs = d_srow_lhs; P.srow_rhs = d_srow_rhs;
    P.n_lrows = n_lrows; P.n_tiles = n_tiles;
    P.lcol = d_lcol; P.lval = d_lval; P.lrow_lhs = d_lrow_lhs; P.lrow_rhs = d_lrow_rhs;
    P.lrow_tile0 = d_lrow_tile0; P.tile_row = d_tile_row; P.tile_begin = d_tile_begin;
    P.tile_end = d_tile_end; P.tile_part = d_tile_part;
    P.lb = d_lb; P.ub = d_ub; P.lb_nxt = d_lb_nxt; P.ub_nxt = d_ub_nxt;
    P.is_cont = d_is_cont; P.chg = d_chg; P.n_chg_words = n_words;
    P.flags = d_flags; P.barrier = d_barrier;
    P.max_rounds = opts.max_rounds;

    finalize_blocks = std::max(1, std::min((n_words + kFinalizeThreads - 1) / kFinalizeThreads, 4 * n_sms));
    int bps = 0;
    GDP_CUDA(megakernel_occupancy(kMegaThreads, &bps));
    mega_grid = std::max(1, bps) * n_sms;
    GDP_CUDA(cudaStreamSynchronize(stream));
    return GDP_OKAY;
}

Context::~Context() {
    if (stream) cudaStreamSynchronize(stream);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (h_flags) cudaFreeHost(h_flags);
    if (stream) cudaStreamDestroy(stream);
}

// Runs the round loop on P.lb/P.ub (already holding the input bounds; nxt
// holding a copy). Fills the round statistics.
GDP_RETCODE Context::run_rounds(cudaStream_t s, gdp_stats *st) {
    RoundFlags init[3];
    std::memset(init, 0, sizeof(init));
    init[0].infeasible_var = INT_MAX;
    GDP_CUDA(cudaMemcpyAsync(P.flags, init, sizeof(init), cudaMemcpyHostToDevice, s));
    int launches = 0;
    GDP_CUDA(launch_check_bounds(P, finalize_blocks, s));
    launches++;
    GDP_CUDA(cudaEventRecord(ev0, s));
    if (opts.sync_type == MEGAKERNEL) {
        GDP_CUDA(cudaMemsetAsync(P.barrier, 0, sizeof(unsigned) * 2, s));
        GDP_CUDA(launch_megakernel(P, mega_grid, kMegaThreads, s));
        launches++;
        GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
        GDP_CUDA(cudaEventRecord(ev1, s));
        GDP_CUDA(cudaStreamSynchronize(s));
    } else {
        GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
        GDP_CUDA(cudaStreamSynchronize(s));
        bool go = !h_flags[0].infeasible;
        for (int r = 1; go && r <= opts.max_rounds; r++) {
            GDP_CUDA(launch_round_begin(P, s));
            GDP_CUDA(launch_split_partial(P, s));
            GDP_CUDA(launch_sell_round(P, s));
            GDP_CUDA(launch_split_cand(P, s));
            GDP_CUDA(launch_finalize(P, finalize_blocks, s));
            launches += 2 + (n_slices > 0) + 2 * (n_tiles > 0);
            GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
            GDP_CUDA(cudaStreamSynchronize(s));
            go = h_flags[0].change && !h_flags[0].infeasible;
        }
        GDP_CUDA(cudaEventRecord(ev1, s));
        GDP_CUDA(cudaStreamSynchronize(s));
    }
    const RoundFlags &f = h_flags[0];
    if (f.error != kErrNone) {
        set_error("device error " + std::to_string(f.error) + " (grid barrier wait exceeded its limit)");
        if (st) st->device_error = f.error;
        return GDP_ERROR;
    }
    if (st) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        st->rounds = f.rounds;
        st->infeasible = f.infeasible;
        st->infeasible_var = f.infeasible ? f.infeasible_var : -1;
        // converged: the last executed round changed nothing, or infeasible
        st->converged = (f.infeasible || !f.change) ? 1 : 0;
        st->device_error = f.error;
        st->kernel_launches = launches;
        st->changed_vars = f.changed_vars;
        st->rows_processed = (long long)f.rounds * rows_nonempty;
        st->nnz_processed = (long long)f.rounds * nnz_rows;
        st->bytes_algorithmic = (double)f.rounds * (12.0 * nnz_rows + 20.0 * rows_nonempty + 36.0 * n);
        st->device_ms = ms;
    }
    return GDP_OKAY;
}

GDP_RETCODE Context::propagate_host(double *lbs, double *ubs, gdp_stats *st) {
    const size_t bytes = sizeof(double) * (size_t)n;
    GDP_CUDA(cudaMemcpyAsync(d_lb, lbs, bytes, cudaMemcpyHostToDevice, stream));
    GDP_CUDA(cudaMemcpyAsync(d_ub, ubs, bytes, cudaMemcpyHostToDevice, stream));
    P.lb = d_lb; P.ub = d_ub;
    GDP_CUDA(cudaMemcpyAsync(d_lb_nxt, d_lb, bytes, cudaMemcpyDeviceToDevice, stream));
    GDP_CUDA(cudaMemcpyAsync(d_ub_nxt, d_ub, bytes, cudaMemcpyDeviceToDevice, stream));
    if (run_rounds(stream, st) != GDP_OKAY) return GDP_ERROR;
    GDP_CUDA(cudaMemcpyAsync(lbs, d_lb, bytes, cudaMemcpyDeviceToHost, stream));
    GDP_CUDA(cudaMemcpyAsync(ubs, d_ub, bytes, cudaMemcpyDeviceToHost, stream));
    GDP_CUDA(cudaStreamSynchronize(stream));
    return GDP_OKAY;
}

GDP_RETCODE Context::propagate_device(double *d_lbs, double *d_ubs, cudaStream_t s, gdp_stats *st) {
    if (!s) s = stream;
    const size_t bytes = sizeof(double) * (size_t)n;
    P.lb = d_lbs; P.ub = d_ubs;
    GDP_CUDA(cudaMemcpyAsync(d_lb_nxt, d_lbs, bytes, cudaMemcpyDeviceToDevice, s));
    GDP_CUDA(cudaMemcpyAsync(d_ub_nxt, d_ubs, bytes, cudaMemcpyDeviceToDevice, s));
    const GDP_RETCODE rc = run_rounds(s, st);
    P.lb = d_lb; P.ub = d_ub;
    return rc;
}

}  // namespace gdp

// gdp_noalloc.cu -- propagation entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: a branch-and-bound solver or a
// framework whose device memory is owned by its own pool (PyTorch's caching
// allocator, a solver's arena) and that propagates thousands of nodes in a
// loop, where cudaMalloc/cudaFree would synchronize the device and fragment
// the pool. gdp_propagate_noalloc serves them: the caller passes the problem
// and the bounds already in device memory, and the working memory the round
// loop needs (next-bound buffers, changed-variable bitmap, round flags) lives
// in one file-scope device array of fixed size, kNoallocMaxVars variables.
//
// That array exists once per GPU that loads this library and stays resident
// until the process exits. Every call shares it and it keeps the last call's
// contents, so each call re-initialises what must start at zero (bitmap,
// flags) and copies the input bounds into the next-bound buffers; two calls
// that overlap on the GPU (different streams or threads at the same time)
// race on it and must be serialized by the caller.
//
// The CSR is checked on the device before any round (row pointers, column
// range, variable types, finite coefficients), so a bad index is reported as
// an error instead of turning into an out-of-range access.
//
// Rows are summed left to right by one thread each with the reference's row
// test (the reference's cpu_omp round function, bit for bit), so results
// equal those of the context path for every row up to the context's
// thread_row_max; longer rows serialize on one thread here.
#include <cuda_runtime.h>

#include <chrono>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>

#include "gdp_context.h"
#include "gdp_device.cuh"

namespace gdp {
namespace {

constexpr int kNoallocMaxVars = 1 << 20;
constexpr int kNoallocWords = kNoallocMaxVars / 32;
constexpr size_t kNoallocBytes =
        2 * sizeof(double) * (size_t)kNoallocMaxVars + sizeof(unsigned) * (size_t)kNoallocWords + 256;
static_assert(sizeof(RoundFlags) + 4 * sizeof(int) <= 256, "flags and input checks fit the reserve");

// [lb_nxt: kNoallocMaxVars doubles][ub_nxt: kNoallocMaxVars doubles][bitmap][flags][input checks]
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

struct NoallocView {
    double *lb_nxt, *ub_nxt;
    unsigned *chg;
    RoundFlags *flags;
    int *bad;  // first offending index per input check (INT_MAX: none), see k_noalloc_validate
};

NoallocView view_of(unsigned char *base) {
    NoallocView v;
    v.lb_nxt = reinterpret_cast<double *>(base);
    v.ub_nxt = v.lb_nxt + kNoallocMaxVars;
    v.chg = reinterpret_cast<unsigned *>(v.ub_nxt + kNoallocMaxVars);
    v.flags = reinterpret_cast<RoundFlags *>(v.chg + kNoallocWords);
    v.bad = reinterpret_cast<int *>(v.flags + 1);
    return v;
}

// Device address of the scratch array, looked up once per device (the host
// symbol g_noalloc_scratch is only a stand-in for it in host code).
std::mutex g_setup_mutex;
unsigned char *g_scratch_addr[64] = {nullptr};

struct Csr {
    int m, n;
    const int *col, *row_ptr, *vartype;
    const double *val, *lhs, *rhs;
    double *lb, *ub;
};

// Input checks of the device CSR, each reading only in-range entries of the
// arrays it checks: bad[0] the first row i with row_ptr[i + 1] < row_ptr[i]
// (-1: row_ptr[0] != 0 or row_ptr[m] != nnz), bad[1] the first non-zero whose
// column is outside [0, n), bad[2] the first variable whose type is not 0, 1
// or 3, bad[3] the first non-finite coefficient.
__global__ void k_noalloc_validate(Csr A, int nnz, NoallocView S) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    if (tid == 0 && (A.row_ptr[0] != 0 || A.row_ptr[A.m] != nnz)) atomicMin(S.bad + 0, -1);
    for (int i = tid; i < A.m; i += nt)
        if (A.row_ptr[i + 1] < A.row_ptr[i]) atomicMin(S.bad + 0, i);
    for (int k = tid; k < nnz; k += nt) {
        const int j = A.col[k];
        if (j < 0 || j >= A.n) atomicMin(S.bad + 1, k);
        if (!isfinite(A.val[k])) atomicMin(S.bad + 3, k);
    }
    for (int j = tid; j < A.n; j += nt) {
        const int t = A.vartype[j];
        if (t != 0 && t != 1 && t != 3) atomicMin(S.bad + 2, j);
    }
}

__global__ void k_noalloc_check(Csr A, NoallocView S) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.n; j += gridDim.x * blockDim.x)
        if (var_infeasible(A.lb[j], A.ub[j])) {
            S.flags->infeasible = 1;
            atomicMin(&S.flags->infeasible_var, j);
        }
}

// One Jacobi round, one thread per row, CSR as given.
__global__ void k_noalloc_round(Csr A, NoallocView S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool tight = false;
    if (i < A.m) {
        const int b = A.row_ptr[i], e = A.row_ptr[i + 1];
        RowActs a;
        acts_init(a);
        for (int k = b; k < e; k++) {
            const int j = A.col[k];
            acts_add(a, A.val[k], A.lb[j], A.ub[j]);
        }
        const double lhs = A.lhs[i], rhs = A.rhs[i];
        if (e > b && row_infeasible(a.minact, a.maxact, a.minact_inf, a.maxact_inf, lhs, rhs))
            atomicMin(&S.flags->infeasible_row, i);
        if (e > b && can_cons_be_tightened(a, lhs, rhs)) {
            const RowCand rc = row_cand(a, lhs, rhs);
            for (int k = b; k < e; k++) {
                const int j = A.col[k];
                bool lt, ut;
                double nl, nu;
                tighten_variable(A.val[k], rc, A.vartype[j] == 3, A.lb[j], A.ub[j], lt, nl, ut, nu);
                if (lt) atomic_max_f64(S.lb_nxt + j, nl);
                if (ut) atomic_min_f64(S.ub_nxt + j, nu);
                if (lt || ut) {
                    atomicOr(S.chg + (j >> 5), 1u << (j & 31));
                    tight = true;
                }
            }
        }
    }
    if (__any_sync(0xffffffffu, tight) && (threadIdx.x & 31) == 0) S.flags->change = 1;
}

__global__ void k_noalloc_finalize(Csr A, NoallocView S, int words) {
    int changed = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0 && S.flags->infeasible_row != INT_MAX) S.flags->infeasible = 1;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x) {
        unsigned bits = S.chg[w];
        if (!bits) continue;
        S.chg[w] = 0u;
        changed += __popc(bits);
        while (bits) {
            const int j = w * 32 + __ffs(bits) - 1;
            bits &= bits - 1;
            const double l = S.lb_nxt[j], u = S.ub_nxt[j];
            A.lb[j] = l;
            A.ub[j] = u;
            if (var_infeasible(l, u)) {
                S.flags->infeasible = 1;
                atomicMin(&S.flags->infeasible_var, j);
            }
        }
    }
    if (changed) atomicAdd(&S.flags->changed_vars, (unsigned long long)changed);
}

__global__ void k_noalloc_round_begin(NoallocView S) {
    S.flags->change = 0;
    S.flags->rounds += 1;
}

#define NA_CUDA(expr)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            set_error(std::string(#expr) + " failed: " + cudaGetErrorString(e_));       \
            return GDP_ERROR;                                                           \
        }                                                                               \
    } while (0)

GDP_RETCODE scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return GDP_ERROR; }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        NA_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_addr[dev];
    return GDP_OKAY;
}

}  // namespace

GDP_RETCODE propagate_noalloc(int m, int n, int nnz, const int *d_col, const int *d_row_ptr,
                              const double *d_val, const double *d_lhs, const double *d_rhs,
                              double *d_lb, double *d_ub, const int *d_vartype, int max_rounds,
                              cudaStream_t s, gdp_stats *st) {
    const auto t0 = std::chrono::steady_clock::now();
    if (st) *st = gdp_stats{};
    if (m < 0 || n < 0 || nnz < 0) { set_error("negative problem size"); return GDP_ERROR; }
    if (n > kNoallocMaxVars) {
        set_error("gdp_propagate_noalloc supports at most " + std::to_string(kNoallocMaxVars) +
                  " variables (its fixed device scratch); got " + std::to_string(n));
        return GDP_ERROR;
    }
    if (m == 0 || n == 0 || nnz == 0) {
        if (st) { st->converged = 1; st->infeasible_var = -1; st->infeasible_row = -1; }
        return GDP_OKAY;
    }
    if (!d_col || !d_row_ptr || !d_val || !d_lhs || !d_rhs || !d_lb || !d_ub || !d_vartype) {
        set_error("null device pointer");
        return GDP_ERROR;
    }
    if (max_rounds <= 0) max_rounds = GDP_MAX_NUM_ROUNDS;
    unsigned char *base = nullptr;
    if (scratch_for_current_device(&base) != GDP_OKAY) return GDP_ERROR;
    const NoallocView S = view_of(base);
    const Csr A{m, n, d_col, d_row_ptr, d_vartype, d_val, d_lhs, d_rhs, d_lb, d_ub};
    const int words = (n + 31) / 32;

    // the input checks first: nothing below indexes with the caller's CSR
    // until they have passed
    const int no_bad[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
    int bad[4];
    NA_CUDA(cudaMemcpyAsync(S.bad, no_bad, sizeof(no_bad), cudaMemcpyHostToDevice, s));
    const int big = m > nnz ? (m > n ? m : n) : (nnz > n ? nnz : n);
    k_noalloc_validate<<<(big + 255) / 256 < 1024 ? (big + 255) / 256 : 1024, 256, 0, s>>>(A, nnz, S);
    NA_CUDA(cudaGetLastError());
    NA_CUDA(cudaMemcpyAsync(bad, S.bad, sizeof(bad), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    if (bad[0] != INT_MAX) {
        set_error(bad[0] < 0 ? std::string("csr_row_ptrs must start at 0 and end at nnz")
                             : "csr_row_ptrs is not monotone (row " + std::to_string(bad[0]) + ")");
        return GDP_ERROR;
    }
    if (bad[1] != INT_MAX) {
        set_error("column index out of range at non-zero " + std::to_string(bad[1]));
        return GDP_ERROR;
    }
    if (bad[2] != INT_MAX) {
        set_error("vartype must be 0, 1 or 3 (variable " + std::to_string(bad[2]) + ")");
        return GDP_ERROR;
    }
    if (bad[3] != INT_MAX) {
        set_error("non-finite coefficient at non-zero " + std::to_string(bad[3]));
        return GDP_ERROR;
    }

    RoundFlags init;
    std::memset(&init, 0, sizeof(init));
    init.infeasible_var = INT_MAX;
    init.infeasible_row = INT_MAX;
    NA_CUDA(cudaMemcpyAsync(S.flags, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemsetAsync(S.chg, 0, sizeof(unsigned) * (size_t)words, s));
    NA_CUDA(cudaMemcpyAsync(S.lb_nxt, d_lb, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    NA_CUDA(cudaMemcpyAsync(S.ub_nxt, d_ub, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    const int vblocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    const int wblocks = (words + 255) / 256 < 1024 ? (words + 255) / 256 : 1024;
    k_noalloc_check<<<vblocks, 256, 0, s>>>(A, S);
    NA_CUDA(cudaGetLastError());
    RoundFlags f;
    NA_CUDA(cudaMemcpyAsync(&f, S.flags, sizeof(f), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    int launches = 1;
    for (int r = 1; !f.infeasible && r <= max_rounds; r++) {
        k_noalloc_round_begin<<<1, 1, 0, s>>>(S);
        k_noalloc_round<<<(m + 127) / 128, 128, 0, s>>>(A, S);
        k_noalloc_finalize<<<wblocks, 256, 0, s>>>(A, S, words);
        NA_CUDA(cudaGetLastError());
        launches += 3;
        NA_CUDA(cudaMemcpyAsync(&f, S.flags, sizeof(f), cudaMemcpyDeviceToHost, s));
        NA_CUDA(cudaStreamSynchronize(s));
        if (!f.change) break;
    }
    if (st) {
        st->rounds = f.rounds;
        st->infeasible = f.infeasible;
        st->infeasible_var = (f.infeasible && f.infeasible_var != INT_MAX) ? f.infeasible_var : -1;
        st->infeasible_row = (f.infeasible && f.infeasible_row != INT_MAX) ? f.infeasible_row : -1;
        st->converged = (f.infeasible || !f.change) ? 1 : 0;
        st->kernel_launches = launches + 1;
        st->changed_vars = f.changed_vars;
        st->rows_processed = (long long)f.rounds * m;
        st->nnz_processed = (long long)f.rounds * nnz;
        st->bytes_algorithmic = (double)f.rounds * (12.0 * nnz + 20.0 * m + 36.0 * n);
        st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return GDP_OKAY;
}

}  // namespace gdp

#pragma GCC visibility push(default)
extern "C" GDP_RETCODE gdp_propagate_noalloc(int n_cons, int n_vars, int nnz, const int *d_csr_col_indices,
                                             const int *d_csr_row_ptrs, const double *d_csr_vals,
                                             const double *d_lhss, const double *d_rhss, double *d_lbs,
                                             double *d_ubs, const int *d_vartypes, int max_rounds,
                                             void *stream, gdp_stats *stats) {
    try {
        return gdp::propagate_noalloc(n_cons, n_vars, nnz, d_csr_col_indices, d_csr_row_ptrs, d_csr_vals,
                                      d_lhss, d_rhss, d_lbs, d_ubs, d_vartypes, max_rounds,
                                      static_cast<cudaStream_t>(stream), stats);
    } catch (const std::exception &e) {
        gdp::set_error(e.what());
        return GDP_ERROR;
    }
}
#pragma GCC visibility pop

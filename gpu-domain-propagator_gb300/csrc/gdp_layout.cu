// gdp_layout.cu -- device-side construction of the layout's element arrays
// from the raw CSR (below), and of the marking index: for every
// variable, the row positions (SELL slot or split-row slot) of the rows it
// appears in, with |a| rounded up (the drift bound's coefficients). This is
// the transpose (CSR -> CSC pattern) that the reference computes with
// cuSPARSE csr2csc on every call (src/kernels/util_kernels.cuh:92-229) and
// uses to mark constraints (src/propagation_methods.cu:3-13).
//
// The column counts and their exclusive scan come from the raw columns
// alone, so they run while the host still bins the rows; the kernels that
// place the elements scatter each one's position into its column's next slot.
// The order of positions inside a column is not defined (it does not matter
// for marking or for the drift sums).
#include <cuda_runtime.h>

#include <climits>

#include "gdp_device.cuh"
#include "gdp_internal.h"

namespace gdp {
namespace {

constexpr int kScanBlock = 1024;

// Counts the raw columns (out-of-range ones skipped: the element checks report them).
__global__ void k_count_raw(const int *__restrict__ col, int nnz, int n, int *cnt) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) {
        const int j = __ldcs(col + k);
        if ((unsigned)j < (unsigned)n) atomicAdd(cnt + j, 1);
    }
}

// Block-level exclusive scan (Hillis-Steele in shared memory; counts fit int).
__global__ void k_scan_blocks(const int *in, int *out, int *block_sums, int n) {
    __shared__ int s[kScanBlock];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        const int t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

// Exclusive scan of the block sums by one block (sequential chunks).
__global__ void k_scan_sums(int *sums, int nb) {
    __shared__ int s[kScanBlock];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < nb; c0 += kScanBlock) {
        const int i = c0 + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < kScanBlock; off <<= 1) {
            const int t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry += s[threadIdx.x];
        __syncthreads();
    }
}

__global__ void k_add_offsets(int *out, const int *block_sums, int n) {
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
}

}  // namespace

int build_marking_counts(const int *col, int nnz, int n, int *var_ptr, int *cursor, int *scratch, cudaStream_t s) {
    const int n1 = n + 1;
    const int nb = (n1 + kScanBlock - 1) / kScanBlock;
    cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)n1, s);
    if (e != cudaSuccess) return (int)e;
    if (nnz > 0) k_count_raw<<<1024, 256, 0, s>>>(col, nnz, n, cursor);
    k_scan_blocks<<<nb, kScanBlock, 0, s>>>(cursor, var_ptr, scratch, n1);
    k_scan_sums<<<1, kScanBlock, 0, s>>>(scratch, nb);
    k_add_offsets<<<nb, kScanBlock, 0, s>>>(var_ptr, scratch, n1);
    e = cudaMemcpyAsync(cursor, var_ptr, sizeof(int) * (size_t)n1, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaGetLastError();
}

// ---- element arrays from the raw CSR -----------------------------------------
// The host decides the layout (row order, slices, split-row tiles: O(m) work)
// and uploads the CSR once; these kernels check the elements (column range,
// finite coefficients), fill the per-position arrays (thread per position)
// and place every element with its FP32 screen copy: SELL slot and
// row-contiguous copy, split-row arrays (block per split row). Padding slots
// of the SELL arrays stay as cleared before.
namespace {
// Element (column c, coefficient v) of row position p into the marking index.
__device__ __forceinline__ void index_element(const LayoutBuild &L, int c, double v, int p) {
    if ((unsigned)c >= (unsigned)L.n) return;  // reported by the element checks
    const int slot = atomicAdd(L.idx_cursor + c, 1);
    L.var_ent[slot] = VarEntry{p, __double2float_ru(fabs(v))};
}

// Places the elements of SELL row positions, each with its FP32 screen copy
// (coef_screen) in both layouts. One-lane rows (positions from g1_begin) go
// thread per row: the threads of a warp hold consecutive rows of one slice,
// so every step k stores 32 consecutive slots. Wider rows go warp per row.
__global__ void __launch_bounds__(256) k_build_sell(LayoutBuild L) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    for (int p = L.g1_begin + tid; p < L.n_srows; p += stride) {
        const int i = L.order[p];
        const int s = L.pos_slice[p];
        const long long base = L.slice_ptr[s] + (p - L.slice_row0[s]);
        const int b = L.row_ptr[i], len = L.row_ptr[i + 1] - b;
        const long long xb = L.xptr[p];
#pragma unroll 4
        for (int k = 0; k < len; k++) {
            const int c = __ldg(L.col + b + k);
            const double v = __ldg(L.val + b + k);
            const float a = coef_screen(v);
            const long long e = base + 32LL * k;
            L.sell_col[e] = c;
            L.sell_val[e] = v;
            L.sell_a32[e] = a;
            L.xcol[xb + k] = c;
            L.xval[xb + k] = v;
            L.xa32[xb + k] = a;
            index_element(L, c, v, p);
        }
    }
    const int lane = threadIdx.x & 31;
    for (int p = tid >> 5; p < L.g1_begin; p += stride >> 5) {
        const int i = L.order[p];
        const int s = L.pos_slice[p];
        const int lg = L.slice_lg[s], g = 1 << lg;
        const int rl = p - L.slice_row0[s];
        const long long base = L.slice_ptr[s] + ((long long)rl << lg);
        const int b = L.row_ptr[i], len = L.row_ptr[i + 1] - b;
        const long long xb = L.xptr[p];
#pragma unroll 2
        for (int k = lane; k < len; k += 32) {
            const int c = __ldg(L.col + b + k);
            const double v = __ldg(L.val + b + k);
            const float a = coef_screen(v);
            const long long e = base + 32LL * (k >> lg) + (k & (g - 1));
            L.sell_col[e] = c;
            L.sell_val[e] = v;
            L.sell_a32[e] = a;
            L.xcol[xb + k] = c;
            L.xval[xb + k] = v;
            L.xa32[xb + k] = a;
            index_element(L, c, v, p);
        }
    }
}

__global__ void __launch_bounds__(256) k_build_positions(LayoutBuild L) {
    const int stride = gridDim.x * blockDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < L.n_srows; p += stride) {
        const int i = L.order[p];
        const int len = L.row_ptr[i + 1] - L.row_ptr[i];
        L.srow_len_out[p] = len;
        L.srow_lhs_out[p] = L.lhs[i];
        L.srow_rhs_out[p] = L.rhs[i];
        L.xptr_out[p] = (int)(L.len_base[len] + (long long)(p - L.len_start[len]) * ((len + 3) & ~3));
    }
    for (int sl = blockIdx.x * blockDim.x + threadIdx.x; sl < L.n_slices; sl += stride)
        for (int p = L.slice_row0[sl]; p < L.slice_row0[sl + 1]; p++) L.pos_slice_out[p] = sl;
}

__global__ void __launch_bounds__(256) k_check_elements(const int *__restrict__ col, const double *__restrict__ val,
                                                        int nnz, int n, int *bad) {
    int bc = INT_MAX, bv = INT_MAX;
    const int stride = gridDim.x * blockDim.x;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += stride) {
        if ((unsigned)__ldcs(col + k) >= (unsigned)n) bc = min(bc, k);
        const long long b = __double_as_longlong(__ldcs(val + k));
        if ((b & 0x7FF0000000000000LL) == 0x7FF0000000000000LL) bv = min(bv, k);  // inf or NaN
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        bc = min(bc, __shfl_xor_sync(0xffffffffu, bc, off));
        bv = min(bv, __shfl_xor_sync(0xffffffffu, bv, off));
    }
    if ((threadIdx.x & 31) == 0) {
        if (bc != INT_MAX) atomicMin(bad, bc);
        if (bv != INT_MAX) atomicMin(bad + 1, bv);
    }
}

__global__ void __launch_bounds__(256) k_build_split(LayoutBuild L) {
    for (int r = blockIdx.x; r < L.n_lrows; r += gridDim.x) {
        const int i = L.split_rows[r];
        const int b = L.row_ptr[i], len = L.row_ptr[i + 1] - b;
        const long long o = L.lrow_ptr[r];
#pragma unroll 4
        for (int k = threadIdx.x; k < len; k += blockDim.x) {
            const double v = __ldg(L.val + b + k);
            const int c = __ldg(L.col + b + k);
            L.lcol[o + k] = c;
            L.lval[o + k] = v;
            L.la32[o + k] = coef_screen(v);
            index_element(L, c, v, L.n_srows + r);
        }
    }
}
}  // namespace

int build_layout_positions(const LayoutBuild &L, int blocks, cudaStream_t s) {
    if (L.n_srows > 0) k_build_positions<<<blocks, 256, 0, s>>>(L);
    return (int)cudaGetLastError();
}

int check_csr_elements(const int *col, const double *val, int nnz, int n, int *bad, int blocks, cudaStream_t s) {
    if (nnz > 0) k_check_elements<<<blocks, 256, 0, s>>>(col, val, nnz, n, bad);
    return (int)cudaGetLastError();
}

int build_layout_elements(const LayoutBuild &L, int blocks, cudaStream_t s) {
    if (L.n_srows > 0) k_build_sell<<<blocks, 256, 0, s>>>(L);
    if (L.n_lrows > 0) k_build_split<<<blocks, 256, 0, s>>>(L);
    return (int)cudaGetLastError();
}

}  // namespace gdp

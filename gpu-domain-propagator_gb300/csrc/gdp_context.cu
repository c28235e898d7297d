// gdp_context.cu -- host side of the propagator: input validation, device
// layout (SELL slices of thread rows, warp tiles of split rows, work items,
// marking index), device buffers and the three round-loop drivers.
//
// Replaces the reference's per-call host driver propagateConstraintsGPUAtomic
// (src/propagators/GPU_propagator.cuh:98-268): uploads, row binning
// (fill_row_blocks, src/kernels/util_kernels.cu:12-62) and the round loops
// (CPU_LOOP :160-204, GPU_LOOP :146-159, MEGAKERNEL :205-255). CUDA errors
// return GDP_ERROR with a message instead of exit() (src/cuda_def.cuh:10-15).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>
#ifdef GDP_BUILD_TIMERS
#include <chrono>
#include <cstdio>
#endif

#ifdef _OPENMP
#include <omp.h>
#endif

#include "gdp_context.h"
#include "gdp_device.cuh"
#include "gdp_learned.h"

namespace gdp {

namespace {
thread_local std::string g_last_error;

// Allocator that leaves the elements of a resized vector uninitialised: the
// layout's per-row host arrays are written in full by parallel loops, and
// zero-filling them first cost a serial pass over megabytes.
template <class T>
struct NoInit : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInit<U>;
    };
    NoInit() = default;
    template <class U>
    NoInit(const NoInit<U> &) {}
    template <class U>
    void construct(U *p) {
        ::new ((void *)p) U;
    }
    template <class U, class... A>
    void construct(U *p, A &&...a) {
        ::new ((void *)p) U(std::forward<A>(a)...);
    }
};
template <class T>
using RawVec = std::vector<T, NoInit<T>>;

// Build stamps, compiled only into a library built with -DGDP_BUILD_TIMERS
// (build.py --build-timers): host wall-clock times of Context::init's
// milestones (ms since it began) and device times of the raw CSR upload and
// the layout kernels, printed to stderr when a build ends. In the plain build
// every call is empty.
struct BuildStamps {
#ifdef GDP_BUILD_TIMERS
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double host[7] = {};
    cudaEvent_t ev[4] = {};  // upload begins / ends (helper stream), layout begins / ends
    void mark(int k) {
        host[k] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    void record(int k, cudaStream_t s) {
        if (!ev[k]) cudaEventCreate(&ev[k]);
        cudaEventRecord(ev[k], s);
    }
    void report() {
        float up = 0.f, start = 0.f, lay = 0.f;
        if (ev[0] && ev[1]) cudaEventElapsedTime(&up, ev[0], ev[1]);
        if (ev[0] && ev[2]) cudaEventElapsedTime(&start, ev[0], ev[2]);
        if (ev[2] && ev[3]) cudaEventElapsedTime(&lay, ev[2], ev[3]);
        fprintf(stderr,
                "gdp build (ms): validated %.2f set-up %.2f binned %.2f joined %.2f launched %.2f queued %.2f "
                "synced %.2f | device: upload %.2f, layout starts %.2f after the upload began, layout %.2f\n",
                host[0], host[1], host[2], host[3], host[4], host[5], host[6], up, start, lay);
    }
    ~BuildStamps() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
#else
    void mark(int) {}
    void record(int, cudaStream_t) {}
    void report() {}
#endif
};
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
namespace {
// Device blocks of released arenas by (device, size). A request takes the
// smallest cached block of its device that is at least as large and at most
// 5/4 of the request. The cache keeps at most kCacheMax bytes; blocks beyond
// that are freed. The object is never destroyed: at exit the CUDA runtime
// may be gone before static destructors run, and the driver reclaims the
// memory anyway.
struct BlockCache {
    std::mutex mu;
    std::multimap<std::pair<int, size_t>, void *> blocks;
    size_t bytes = 0;
};
constexpr size_t kCacheMax = size_t(32) << 30;
BlockCache &block_cache() {
    static BlockCache *c = new BlockCache;
    return *c;
}
}  // namespace

void release_cached_memory() {
    BlockCache &c = block_cache();
    std::lock_guard<std::mutex> g(c.mu);
    int cur = 0;
    cudaGetDevice(&cur);
    for (const auto &kv : c.blocks) {
        cudaSetDevice(kv.first.first);
        cudaFree(kv.second);
    }
    cudaSetDevice(cur);
    cudaGetLastError();
    c.blocks.clear();
    c.bytes = 0;
}

Arena::~Arena() { release(); }

void Arena::release() {
    if (blocks.empty()) return;
    // a block may still be read by work on any stream of its device (the
    // device-pointer entry points take the caller's stream): wait for the
    // device, as cudaFree would
    int cur = 0;
    cudaGetDevice(&cur);
    int synced = -1;
    for (const Block &b : blocks)
        if (b.dev != synced) {
            cudaSetDevice(b.dev);
            cudaDeviceSynchronize();
            synced = b.dev;
        }
    cudaSetDevice(cur);
    cudaGetLastError();
    BlockCache &c = block_cache();
    std::lock_guard<std::mutex> g(c.mu);
    for (const Block &b : blocks) {
        if (c.bytes + b.bytes <= kCacheMax) {
            c.blocks.emplace(std::make_pair(b.dev, b.bytes), b.p);
            c.bytes += b.bytes;
        } else {
            cudaFree(b.p);
        }
    }
    blocks.clear();
}

void *Arena::alloc_bytes(size_t bytes) {
    bytes = (std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    {
        BlockCache &c = block_cache();
        std::lock_guard<std::mutex> g(c.mu);
        auto it = c.blocks.lower_bound(std::make_pair(dev, bytes));
        if (it != c.blocks.end() && it->first.first == dev && it->first.second - bytes <= bytes / 4) {
            const Block blk{it->second, it->first.second, dev};
            c.blocks.erase(it);
            c.bytes -= blk.bytes;
            blocks.push_back(blk);
            return blk.p;
        }
    }
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {  // the cache may hold the memory: free it, retry once
        cudaGetLastError();
        release_cached_memory();
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    blocks.push_back(Block{p, bytes, dev});
    return p;
}

// ---------------------------------------------------------------------------
// The checks that make the raw arrays safe to copy: sizes, pointers and the
// row pointer's end points.
static GDP_RETCODE validate_shape(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                                  const int *vartype) {
    if (m < 0 || n < 0 || nnz < 0) { set_error("negative problem size"); return GDP_ERROR; }
    if (!col || !row_ptr || !val || !vartype) { set_error("null input array"); return GDP_ERROR; }
    if (row_ptr[0] != 0 || row_ptr[m] != nnz) {
        set_error("csr_row_ptrs must start at 0 and end at nnz");
        return GDP_ERROR;
    }
    return GDP_OKAY;
}

GDP_RETCODE validate_csr(int m, int n, int nnz, const int *col, const int *row_ptr,
                         const double *val, const int *vartype) {
    if (validate_shape(m, n, nnz, col, row_ptr, val, vartype) != GDP_OKAY) return GDP_ERROR;
    int bad_row = INT_MAX, bad_var = INT_MAX;
#pragma omp parallel for reduction(min : bad_row) schedule(static)
    for (int i = 0; i < m; i++)
        if (row_ptr[i + 1] < row_ptr[i]) bad_row = std::min(bad_row, i);
    if (bad_row != INT_MAX) { set_error("csr_row_ptrs is not monotone"); return GDP_ERROR; }
#pragma omp parallel for reduction(min : bad_var) schedule(static)
    for (int j = 0; j < n; j++)
        if (vartype[j] != 0 && vartype[j] != 1 && vartype[j] != 3) bad_var = std::min(bad_var, j);
    if (bad_var != INT_MAX) {
        set_error("vartype must be 0, 1 or 3 (variable " + std::to_string(bad_var) + ")");
        return GDP_ERROR;
    }
    return GDP_OKAY;
}

// The element checks (column range, finite coefficients) run on the device
// over the uploaded raw CSR; this turns their result into the error.
static GDP_RETCODE element_error(const int bad[2]) {
    if (bad[0] != INT_MAX) {
        set_error("column index out of range at non-zero " + std::to_string(bad[0]));
        return GDP_ERROR;
    }
    if (bad[1] != INT_MAX) {
        set_error("non-finite coefficient at non-zero " + std::to_string(bad[1]));
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
    if (opts.thread_row_max <= 0) opts.thread_row_max = 32;
    if (opts.split_tile <= 0) opts.split_tile = 1024;
    if (opts.use_marking < 0) opts.use_marking = 1;
    if (opts.thread_row_max > (1 << 20)) opts.thread_row_max = 1 << 20;
    if (opts.split_tile > (1 << 24)) opts.split_tile = 1 << 24;
    if (opts.sync_type < CPU_LOOP || opts.sync_type > MEGAKERNEL) {
        set_error("Unknown sync type");
        return GDP_ERROR;
    }
    if (opts.cta_threads == 0) opts.cta_threads = 256;
    if (opts.cta_threads != 128 && opts.cta_threads != 256 && opts.cta_threads != 512) {
        set_error("cta_threads must be 128, 256 or 512");
        return GDP_ERROR;
    }
    if (!lhs || !rhs) { set_error("null lhs/rhs"); return GDP_ERROR; }
    BuildStamps stamps;
    if (validate_csr(m, n, nnz, col, row_ptr, val, vartype) != GDP_OKAY) return GDP_ERROR;  // host part
    stamps.mark(0);

    GDP_CUDA(cudaSetDevice(opts.device));
    cudaGetLastError();  // every call below is checked; start from a clean error state
    GDP_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    GDP_CUDA(cudaEventCreate(&ev0));
    GDP_CUDA(cudaEventCreate(&ev1));
    GDP_CUDA(cudaMallocHost(&h_flags, sizeof(RoundFlags) * 3));
    int sms = 0;
    GDP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opts.device));
    n_sms = sms;
    int pageable = 0;
    GDP_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, opts.device));
    host_direct = pageable == 1;

    // The raw CSR goes up from a helper thread, on a stream of its own, while
    // this thread bins the rows: a copy from pageable memory returns only
    // once its source has been staged, so issuing it here would serialise
    // the two. This thread makes no CUDA call until the row layout is
    // decided (the driver would hold it while the copy runs). The helper
    // leaves once the copies are queued; the layout build that reads them
    // waits for them on the device (an event), after the join. The element
    // checks (column range, finite coefficients) run on the device over the
    // copies.
    stamps.mark(1);
    Arena raw;  // raw CSR and row sides, released when the build is done
    int *dcol = nullptr, *drp = nullptr;
    double *dval = nullptr, *dlhs = nullptr, *drhs = nullptr;
    std::string up_err;
    struct UploadStream {  // the helper's stream and its completion event
        cudaStream_t s = nullptr;
        cudaEvent_t done = nullptr;
        ~UploadStream() {
            if (s) cudaStreamSynchronize(s);  // before the raw buffers can be freed
            if (done) cudaEventDestroy(done);
            if (s) cudaStreamDestroy(s);
        }
    } ups;
    // marking index (variable -> row positions, |a| rounded up): the helper
    // counts the columns as soon as they are up; the layout kernels fill it
    const size_t n1 = (size_t)n + 1;
    int *vp = (int *)arena.alloc_bytes(sizeof(int) * n1);
    VarEntry *vent = (VarEntry *)arena.alloc_bytes(sizeof(VarEntry) * (size_t)std::max(nnz, 1));
    int *vcur = (int *)raw.alloc_bytes(sizeof(int) * n1);
    int *vscan = (int *)raw.alloc_bytes(sizeof(int) * ((n1 + 1023) / 1024 + 1));
    if (!vp || !vent || !vcur || !vscan) {
        set_error("device allocation failed (marking index)");
        return GDP_ERROR;
    }
    struct Joined {
        std::thread t;
        ~Joined() {
            if (t.joinable()) t.join();
        }
    } uploader;  // declared after everything the thread touches: joined first
    uploader.t = std::thread([&, dev = opts.device] {
        auto fail = [&](const char *what, cudaError_t e) {
            up_err = std::string(what) + ": " + cudaGetErrorString(e);
            cudaGetLastError();
        };
        cudaError_t e = cudaSetDevice(dev);
        if (e != cudaSuccess) return fail("cudaSetDevice", e);
        const size_t nz = (size_t)std::max(nnz, 1);
        dcol = (int *)raw.alloc_bytes(sizeof(int) * nz);
        dval = (double *)raw.alloc_bytes(sizeof(double) * nz);
        drp = (int *)raw.alloc_bytes(sizeof(int) * ((size_t)m + 1));
        dlhs = (double *)raw.alloc_bytes(sizeof(double) * (size_t)std::max(m, 1));
        drhs = (double *)raw.alloc_bytes(sizeof(double) * (size_t)std::max(m, 1));
        if (!dcol || !dval || !drp || !dlhs || !drhs) {
            up_err = "device allocation failed (raw CSR)";
            return;
        }
        e = cudaStreamCreateWithFlags(&ups.s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return fail("cudaStreamCreate", e);
        e = cudaEventCreateWithFlags(&ups.done, cudaEventDisableTiming);
        if (e != cudaSuccess) return fail("cudaEventCreate", e);
        cudaStream_t us = ups.s;
        stamps.record(0, us);
        if (nnz) e = cudaMemcpyAsync(dcol, col, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, us);
        if (e == cudaSuccess && nnz)
            e = cudaMemcpyAsync(dval, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, us);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(drp, row_ptr, sizeof(int) * ((size_t)m + 1), cudaMemcpyHostToDevice, us);
        if (e == cudaSuccess && m) e = cudaMemcpyAsync(dlhs, lhs, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice, us);
        if (e == cudaSuccess && m) e = cudaMemcpyAsync(drhs, rhs, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice, us);
        stamps.record(1, us);
        if (e == cudaSuccess) e = (cudaError_t)build_marking_counts(dcol, nnz, n, vp, vcur, vscan, us);
        if (e == cudaSuccess) e = cudaEventRecord(ups.done, us);
        if (e != cudaSuccess) fail("raw CSR upload", e);
    });

    // host threads while the helper runs: one core stays free for it, so
    // that no parallel region waits for a descheduled thread
#ifdef _OPENMP
    const int host_threads = std::max(1, omp_get_max_threads() - 1);
#else
    const int host_threads = 1;
#endif
    // ---- row binning (SELL-g) ----
    // g = 1 for rows up to thread_row_max; g = smallest power of two >= len/32
    // (2..32) up to split_tile; longer rows are split into warp tiles.
    const int Lt = opts.thread_row_max, Ls = std::max(opts.split_tile, Lt);
    auto lanes_of = [&](int L) {
        if (L <= Lt) return 1;
        int g = 2;
        while (g < 32 && g * 32 < L) g <<= 1;
        return g;
    };
    std::unique_ptr<int[]> len(new int[std::max(m, 1)]);
    int lmax = 0;  // longest SELL row
#pragma omp parallel for reduction(max : lmax) schedule(static) num_threads(host_threads)
    for (int i = 0; i < m; i++) {
        len[i] = row_ptr[i + 1] - row_ptr[i];
        if (len[i] <= Ls) lmax = std::max(lmax, len[i]);
    }
    // SELL rows (1..Ls non-zeros) by lanes per row (widest first), then length
    // (longest first), stable: lanes_of never decreases with the length, so
    // this is a counting sort by length, longest first -- run in parallel over
    // contiguous row chunks (per-chunk histograms keep it stable). Split rows
    // (longer than Ls) are collected in row order and sorted by length.
    // pos_row: the original row of every position -- SELL positions first (the
    // row order the layout is built from), then the split rows; uploaded as is
    RawVec<int> pos_row((size_t)std::max(m, 1));
    std::vector<int> split_rows;
    // per SELL row length L: first position, and first element of the
    // row-contiguous copy (rows of one length are consecutive positions)
    std::vector<int> len_start((size_t)lmax + 1, 0);
    std::vector<long long> len_base((size_t)lmax + 1, 0);
    long long x_elems = 0;  // elements of the row-contiguous copy
    int n_sell_rows = 0;
    {
#ifdef _OPENMP
        const int nt = lmax <= (1 << 16) ? std::min(host_threads, 64) : 1;
#else
        const int nt = 1;
#endif
        const size_t W = (size_t)lmax + 1;  // keys 0..lmax (0: empty rows, skipped)
        std::vector<int> hist((size_t)nt * W, 0);
        std::vector<int> nsplit(nt + 1, 0);
#pragma omp parallel num_threads(nt)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            const int i0 = (int)((long long)m * t / nt), i1 = (int)((long long)m * (t + 1) / nt);
            int *h = &hist[(size_t)t * W];
            for (int i = i0; i < i1; i++) {
                if (len[i] > Ls) nsplit[t + 1]++;
                else h[len[i]]++;
            }
        }
        // offsets: longer rows first; within a length, chunks in row order
        int acc = 0;
        for (int L = lmax; L >= 1; L--) {
            len_start[L] = acc;
            len_base[L] = x_elems;
            for (int t = 0; t < nt; t++) {
                const int c = hist[(size_t)t * W + L];
                hist[(size_t)t * W + L] = acc;
                acc += c;
            }
            x_elems += (long long)(acc - len_start[L]) * ((L + 3) & ~3);  // rows start on 4-element boundaries
        }
        for (int t = 0; t < nt; t++) nsplit[t + 1] += nsplit[t];
        n_sell_rows = acc;
        split_rows.resize(nsplit[nt]);
#pragma omp parallel num_threads(nt)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            const int i0 = (int)((long long)m * t / nt), i1 = (int)((long long)m * (t + 1) / nt);
            int *h = &hist[(size_t)t * W];
            int sp = nsplit[t];
            for (int i = i0; i < i1; i++) {
                if (len[i] > Ls) split_rows[sp++] = i;
                else if (len[i] > 0) pos_row[h[len[i]]++] = i;
            }
        }
    }
    std::stable_sort(split_rows.begin(), split_rows.end(), [&](int a, int b) { return len[a] > len[b]; });
    const int ns = n_sell_rows;
    const int *order = pos_row.data();  // row position -> original row

    n_srows = ns;
    // slices: the rows of one lanes-per-row class are consecutive positions;
    // a class of g lanes is cut into slices of 32 / g rows, each as wide as
    // its first (longest) row
    std::vector<long long> slice_ptr;
    std::vector<int> slice_row0, slice_lg;
    int g1_begin = ns;  // first position of the one-lane rows
    {
        int cls_lo[6], cls_hi[6], cls_first[6];
        for (int c = 0; c < 6; c++) { cls_lo[c] = 0; cls_hi[c] = 0; }
        for (int p = 0; p < ns;) {  // class boundaries: binary search on the sorted lengths
            const int g = lanes_of(len[order[p]]);
            int lg = 0;
            while ((1 << lg) < g) lg++;
            int lo = p, hi = ns;  // first position of a smaller class
            while (lo < hi) {
                const int mid = lo + (hi - lo) / 2;
                if (lanes_of(len[order[mid]]) == g) lo = mid + 1;
                else hi = mid;
            }
            cls_lo[lg] = p;
            cls_hi[lg] = lo;
            p = lo;
        }
        if (cls_hi[0] > cls_lo[0]) g1_begin = cls_lo[0];
        int nsl = 0;
        for (int lg = 5; lg >= 0; lg--) {
            cls_first[lg] = nsl;
            const int per = 32 >> lg;
            nsl += (cls_hi[lg] - cls_lo[lg] + per - 1) / per;
        }
        slice_row0.resize((size_t)nsl + 1);
        slice_lg.resize((size_t)std::max(nsl, 1), 0);
        slice_ptr.resize((size_t)nsl + 1);
        std::vector<long long> width((size_t)std::max(nsl, 1), 0);
        for (int lg = 5; lg >= 0; lg--) {
            const int per = 32 >> lg, g = 1 << lg, c0 = cls_lo[lg], c1 = cls_hi[lg];
            const int k_n = (c1 - c0 + per - 1) / per;
#pragma omp parallel for schedule(static) num_threads(host_threads)
            for (int k = 0; k < k_n; k++) {
                const int s = cls_first[lg] + k, r0 = c0 + k * per;
                slice_row0[s] = r0;
                slice_lg[s] = lg;
                width[s] = (len[order[r0]] + g - 1) / g;
            }
        }
        slice_row0[nsl] = ns;
        slice_ptr[0] = 0;
        for (int s = 0; s < nsl; s++) slice_ptr[s + 1] = slice_ptr[s] + 32LL * width[s];
        n_slices = nsl;
    }
    sell_elems = slice_ptr[n_slices];
    // per row position (length, sides, first element of the row-contiguous
    // copy, slice): built on the device from the row order
    // split rows: CSR-contiguous, warp tiles of split_tile non-zeros
    n_lrows = (int)split_rows.size();
    std::vector<long long> lrow_ptr(n_lrows + 1, 0);
    std::vector<int> lrow_tile0(n_lrows + 1, 0);
    std::vector<double> lrow_lhs(std::max(n_lrows, 1)), lrow_rhs(std::max(n_lrows, 1));
    std::vector<int> tile_row, tile_begin, tile_end;
    {  // element and tile offsets (prefix sums), then the row sides and tiles in parallel
        const long long tl = opts.split_tile;
        for (int r = 0; r < n_lrows; r++) {
            const int L = len[split_rows[r]];
            lrow_ptr[r + 1] = lrow_ptr[r] + L;
            lrow_tile0[r + 1] = lrow_tile0[r] + (int)((L + tl - 1) / tl);
        }
        n_tiles = lrow_tile0[n_lrows];
        tile_row.resize(n_tiles);
        tile_begin.resize(n_tiles);
        tile_end.resize(n_tiles);
#pragma omp parallel for schedule(static) num_threads(host_threads)
        for (int r = 0; r < n_lrows; r++) {
            const int i = split_rows[r];
            lrow_lhs[r] = lhs[i];
            lrow_rhs[r] = rhs[i];
            int t = lrow_tile0[r];
            for (long long b = lrow_ptr[r]; b < lrow_ptr[r + 1]; b += tl, t++) {
                tile_row[t] = r;
                tile_begin[t] = (int)b;
                tile_end[t] = (int)std::min(b + tl, lrow_ptr[r + 1]);
            }
        }
    }
    const long long lnnz = lrow_ptr[n_lrows];
    // work items of the activity phase, heaviest first (slices: 32 x width non-zeros)
    std::vector<int> items;
    items.reserve((size_t)n_slices + n_tiles);
    {
        std::vector<std::pair<long long, int>> cost;
        cost.reserve((size_t)n_slices + n_tiles);
        long long wmax = 0;
        for (int s = 0; s < n_slices; s++) cost.emplace_back(slice_ptr[s + 1] - slice_ptr[s], s);
        for (int t = 0; t < n_tiles; t++) cost.emplace_back((long long)(tile_end[t] - tile_begin[t]), -t - 1);
        for (auto &c : cost) wmax = std::max(wmax, c.first);
        if (wmax <= (1 << 20)) {  // stable counting sort, heaviest first
            std::vector<int> start((size_t)wmax + 2, 0);
            for (auto &c : cost) start[c.first]++;
            int acc = 0;
            for (long long w = wmax; w >= 0; w--) {
                const int k = start[w];
                start[w] = acc;
                acc += k;
            }
            items.resize(cost.size());
            for (auto &c : cost) items[start[c.first]++] = c.second;
        } else {
            std::stable_sort(cost.begin(), cost.end(),
                             [](const std::pair<long long, int> &a, const std::pair<long long, int> &b) {
                                 return a.first > b.first;
                             });
            for (auto &c : cost) items.push_back(c.second);
        }
    }
    // ---- upload ----
    auto up = [&](const void *src, size_t bytes) -> void * {
        void *d = arena.alloc_bytes(bytes);
        if (!d) return nullptr;
        if (bytes && cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, stream) != cudaSuccess)
            return nullptr;
        return d;
    };
#define GDP_UP(dst, T, vec)                                                                         \
    do {                                                                                           \
        dst = (T *)up((vec).data(), sizeof((vec)[0]) * (vec).size());                              \
        if (!dst) { set_error("device allocation/upload failed for " #vec); return GDP_ERROR; }     \
    } while (0)
    std::memset(&P, 0, sizeof(P));
    P.n = n;
    P.n_srows = n_srows;
    P.n_slices = n_slices;
    GDP_UP(P.slice_ptr, const long long, slice_ptr);
    GDP_UP(P.slice_row0, const int, slice_row0);
    GDP_UP(P.slice_lg, const int, slice_lg);
    stamps.mark(2);
    int *d_srow_len = (int *)arena.alloc_bytes(sizeof(int) * (size_t)std::max(ns, 1));
    int *d_xptr = (int *)arena.alloc_bytes(sizeof(int) * (size_t)std::max(ns, 1));
    int *d_pos_slice = (int *)arena.alloc_bytes(sizeof(int) * (size_t)std::max(ns, 1));
    double *d_srow_lhs = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(ns, 1));
    double *d_srow_rhs = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(ns, 1));
    if (!d_srow_len || !d_xptr || !d_pos_slice || !d_srow_lhs || !d_srow_rhs) {
        set_error("device allocation failed (row positions)");
        return GDP_ERROR;
    }
    P.srow_len = d_srow_len;
    P.xptr = d_xptr;
    P.pos_slice = d_pos_slice;
    P.srow_lhs = d_srow_lhs;
    P.srow_rhs = d_srow_rhs;
    P.n_lrows = n_lrows;
    P.n_tiles = n_tiles;
    GDP_UP(P.lrow_lhs, const double, lrow_lhs);
    GDP_UP(P.lrow_rhs, const double, lrow_rhs);
    GDP_UP(P.lrow_tile0, const int, lrow_tile0);
    if (tile_row.empty()) { tile_row.push_back(0); tile_begin.push_back(0); tile_end.push_back(0); }
    GDP_UP(P.tile_row, const int, tile_row);
    GDP_UP(P.tile_begin, const int, tile_begin);
    GDP_UP(P.tile_end, const int, tile_end);
    // The device builds the layout and then the marking index while this
    // thread prepares the rest (row origins, work lists, variable types) and
    // sends it up on the helper's stream; one synchronisation at the end, then
    // the element checks' verdict.
    Arena tmp;  // the row maps, freed when the build is done
    int *hbad = reinterpret_cast<int *>(h_flags);  // pinned: the checks' verdict comes back asynchronously
    {  // element arrays: the raw CSR goes up once and the device places every
       // element (SELL slots, row-contiguous copy, split rows) together with
       // its FP32 screen copy
        const size_t n_sell = (size_t)std::max<long long>(sell_elems, 1);
        const size_t n_x = (size_t)std::max<long long>(x_elems, 1);
        const size_t n_l = (size_t)std::max<long long>(lnnz, 1);
        int *sc = (int *)arena.alloc_bytes(sizeof(int) * n_sell);
        double *sv = (double *)arena.alloc_bytes(sizeof(double) * n_sell);
        int *xc = (int *)arena.alloc_bytes(sizeof(int) * n_x);
        double *xv = (double *)arena.alloc_bytes(sizeof(double) * n_x);
        int *lc = (int *)arena.alloc_bytes(sizeof(int) * n_l);
        double *lv = (double *)arena.alloc_bytes(sizeof(double) * n_l);
        float *sa = (float *)arena.alloc_bytes(sizeof(float) * n_sell);
        float *xa = (float *)arena.alloc_bytes(sizeof(float) * n_x);
        float *la = (float *)arena.alloc_bytes(sizeof(float) * n_l);
        if (!sc || !sv || !xc || !xv || !lc || !lv || !sa || !xa || !la) {
            set_error("device allocation failed (layout element arrays)");
            return GDP_ERROR;
        }
        GDP_CUDA(cudaMemsetAsync(sc, 0, sizeof(int) * n_sell, stream));  // padding slots
        GDP_CUDA(cudaMemsetAsync(sv, 0, sizeof(double) * n_sell, stream));
        GDP_CUDA(cudaMemsetAsync(sa, 0, sizeof(float) * n_sell, stream));
        GDP_CUDA(cudaMemsetAsync(xc, 0, sizeof(int) * n_x, stream));  // row padding of the copy
        GDP_CUDA(cudaMemsetAsync(xv, 0, sizeof(double) * n_x, stream));
        GDP_CUDA(cudaMemsetAsync(xa, 0, sizeof(float) * n_x, stream));
        int *dord = (int *)tmp.alloc_bytes(sizeof(int) * (size_t)std::max(ns, 1));
        int *dspl = (int *)tmp.alloc_bytes(sizeof(int) * (size_t)std::max(n_lrows, 1));
        long long *dlrp = (long long *)tmp.alloc_bytes(sizeof(long long) * ((size_t)n_lrows + 1));
        int *dls = (int *)tmp.alloc_bytes(sizeof(int) * len_start.size());
        long long *dlb = (long long *)tmp.alloc_bytes(sizeof(long long) * len_base.size());
        int *dbad = (int *)tmp.alloc_bytes(sizeof(int) * 2);
        if (!dord || !dspl || !dlrp || !dls || !dlb || !dbad) {
            set_error("device allocation failed (row maps)");
            return GDP_ERROR;
        }
        uploader.t.join();
        stamps.mark(3);
        if (!up_err.empty()) {
            set_error(up_err);
            return GDP_ERROR;
        }
        GDP_CUDA(cudaStreamWaitEvent(stream, ups.done, 0));
        stamps.record(2, stream);
        if (ns) GDP_CUDA(cudaMemcpyAsync(dord, order, sizeof(int) * (size_t)ns, cudaMemcpyHostToDevice, stream));
        if (n_lrows)
            GDP_CUDA(cudaMemcpyAsync(dspl, split_rows.data(), sizeof(int) * (size_t)n_lrows, cudaMemcpyHostToDevice,
                                     stream));
        GDP_CUDA(cudaMemcpyAsync(dlrp, lrow_ptr.data(), sizeof(long long) * ((size_t)n_lrows + 1),
                                 cudaMemcpyHostToDevice, stream));
        GDP_CUDA(cudaMemcpyAsync(dls, len_start.data(), sizeof(int) * len_start.size(), cudaMemcpyHostToDevice,
                                 stream));
        GDP_CUDA(cudaMemcpyAsync(dlb, len_base.data(), sizeof(long long) * len_base.size(), cudaMemcpyHostToDevice,
                                 stream));
        const int no_bad[2] = {INT_MAX, INT_MAX};
        GDP_CUDA(cudaMemcpyAsync(dbad, no_bad, sizeof(no_bad), cudaMemcpyHostToDevice, stream));
        GDP_CUDA(check_csr_elements(dcol, dval, nnz, n, dbad, 8 * n_sms, stream));
        LayoutBuild L;
        L.col = dcol; L.row_ptr = drp; L.val = dval;
        L.n_srows = ns; L.order = dord; L.pos_slice = P.pos_slice; L.slice_row0 = P.slice_row0;
        L.slice_lg = P.slice_lg; L.xptr = P.xptr; L.slice_ptr = P.slice_ptr;
        L.sell_col = sc; L.xcol = xc; L.sell_val = sv; L.xval = xv; L.sell_a32 = sa; L.xa32 = xa;
        L.g1_begin = g1_begin; L.la32 = la;
        L.n_lrows = n_lrows; L.split_rows = dspl; L.lrow_ptr = dlrp; L.lcol = lc; L.lval = lv;
        L.lhs = dlhs; L.rhs = drhs; L.len_start = dls; L.len_base = dlb; L.n_slices = n_slices;
        L.srow_len_out = d_srow_len; L.xptr_out = d_xptr; L.pos_slice_out = d_pos_slice;
        L.srow_lhs_out = d_srow_lhs; L.srow_rhs_out = d_srow_rhs;
        L.idx_cursor = vcur; L.var_ent = vent; L.n = n;
        // the layout build uses columns as indices only for the marking
        // index, which skips columns out of range, so it runs before the
        // element checks' verdict is read
        GDP_CUDA(build_layout_positions(L, 8 * n_sms, stream));
        GDP_CUDA(build_layout_elements(L, 8 * n_sms, stream));
        stamps.record(3, stream);
        stamps.mark(4);
        GDP_CUDA(cudaMemcpyAsync(hbad, dbad, sizeof(int) * 2, cudaMemcpyDeviceToHost, stream));
        P.sell_col = sc; P.sell_val = sv; P.sell_a32 = sa;
        P.xcol = xc; P.xval = xv; P.xa32 = xa;
        P.lcol = lc; P.lval = lv; P.la32 = la;
    }
    vec_blocks = std::max(1, std::min((std::max(n, std::max(ns + n_lrows, 1)) + 255) / 256, 8 * n_sms));
    // the marking index (also used by node batches when this context's rounds
    // never mark) was filled with the layout
    P.var_ptr = vp;
    P.var_ent = vent;
    // the rest goes up on the helper's stream while the device builds
    auto up_aux = [&](const void *src, size_t bytes) -> void * {
        void *d = arena.alloc_bytes(bytes);
        if (!d) return nullptr;
        if (bytes && cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, ups.s) != cudaSuccess) return nullptr;
        return d;
    };
#define GDP_UP_AUX(dst, T, vec)                                                                     \
    do {                                                                                           \
        dst = (T *)up_aux((vec).data(), sizeof((vec)[0]) * (vec).size());                          \
        if (!dst) { set_error("device allocation/upload failed for " #vec); return GDP_ERROR; }     \
    } while (0)
    // row-side infeasibility names a position's original row: the split rows
    // follow the SELL positions (the row order uploaded above is staged already)
    std::copy(split_rows.begin(), split_rows.end(), pos_row.begin() + ns);
    if (ns + n_lrows == 0) pos_row[0] = 0;
    P.pos_row = (const int *)up_aux(pos_row.data(), sizeof(int) * (size_t)std::max(ns + n_lrows, 1));
    if (!P.pos_row) { set_error("device allocation/upload failed for pos_row"); return GDP_ERROR; }
    std::vector<int> mtiles;
    for (int r = 0; r < n_lrows; r++)
        if (lrow_tile0[r + 1] - lrow_tile0[r] > 1)
            for (int t = lrow_tile0[r]; t < lrow_tile0[r + 1]; t++) mtiles.push_back(t);
    P.n_mtiles = (int)mtiles.size();
    if (mtiles.empty()) mtiles.push_back(0);
    GDP_UP_AUX(P.mtiles, const int, mtiles);
    P.n_items = (int)items.size();
    if (items.empty()) items.push_back(0);
    GDP_UP_AUX(P.items, const int, items);
    P.use_marking = opts.use_marking < 0 ? 1 : (opts.use_marking > 2 ? 2 : opts.use_marking);
    // adaptive marking: mark when a round tightened fewer bounds than 1/16 of the variables
    P.mark_threshold = (unsigned)std::max(1, n / 16);
    RawVec<unsigned char> is_cont((size_t)std::max(n, 1));
    is_cont[0] = 0;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++) is_cont[j] = vartype[j] == GDP_CONTINUOUS ? 1 : 0;
    GDP_UP_AUX(P.is_cont, const unsigned char, is_cont);
#undef GDP_UP_AUX
#undef GDP_UP
    const int npos = std::max(ns + n_lrows, 1);
    const int n_words = (n + 31) / 32;
    P.tile_part = (TilePart *)arena.alloc_bytes(sizeof(TilePart) * (size_t)std::max(n_tiles, 1));
    P.tile_scr = (TileScr *)arena.alloc_bytes(sizeof(TileScr) * (size_t)std::max(n_tiles, 1));
    // deferred exact pass: per-class row queues (classes are contiguous position ranges)
    P.defer_exact = 1;
    for (int c = 0; c < 6; c++) { P.cls_begin[c] = 0; P.cls_end[c] = 0; }
    for (int sl = n_slices - 1; sl >= 0; sl--) P.cls_begin[slice_lg[sl]] = slice_row0[sl];
    for (int sl = 0; sl < n_slices; sl++) P.cls_end[slice_lg[sl]] = slice_row0[sl + 1];
    P.xrow = (XRow *)arena.alloc_bytes(sizeof(XRow) * (size_t)std::max(ns, 1));
    P.xctr = (unsigned *)arena.alloc_bytes(sizeof(unsigned) * 32);
    P.row_exact = (int *)arena.alloc_bytes(sizeof(int) * (size_t)std::max(n_lrows, 1));
    P.lrow_margin = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n_lrows, 1));
    P.lrow_drift = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n_lrows, 1));
    P.lrow_skip = (int *)arena.alloc_bytes(sizeof(int) * (size_t)std::max(n_lrows, 1));
    P.mark = (int *)arena.alloc_bytes(sizeof(int) * (size_t)npos);
    P.bnd = (double2 *)arena.alloc_bytes(sizeof(double2) * (size_t)std::max(n, 1));
    P.bnd_nxt = (double2 *)arena.alloc_bytes(sizeof(double2) * (size_t)std::max(n, 1));
    P.bnd32 = (float2 *)arena.alloc_bytes(sizeof(BndScr) * (size_t)std::max(n, 1));  // stamped records
    P.chg = (unsigned *)arena.alloc_bytes(sizeof(unsigned) * (size_t)std::max(n_words, 1));
    P.n_chg_words = n_words;
    P.flags = (RoundFlags *)arena.alloc_bytes(sizeof(RoundFlags) * 3);
    P.barrier = (unsigned *)arena.alloc_bytes(sizeof(unsigned) * 2);
    P.queue = (unsigned *)arena.alloc_bytes(sizeof(unsigned) * 8);
    P.max_rounds = opts.max_rounds;
    P.spin_limit = opts.barrier_wait_kcycles > 0 ? 1000LL * opts.barrier_wait_kcycles : 4000000000LL;
    d_lb = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n, 1));
    d_ub = (double *)arena.alloc_bytes(sizeof(double) * (size_t)std::max(n, 1));
    if (!P.tile_part || !P.tile_scr || !P.row_exact || !P.lrow_margin || !P.lrow_drift || !P.lrow_skip || !P.xrow || !P.xctr || !P.mark || !P.bnd || !P.bnd_nxt || !P.bnd32 || !P.chg || !P.flags || !P.barrier || !P.queue ||
        !d_lb || !d_ub) {
        set_error("device allocation failed");
        return GDP_ERROR;
    }

    if (set_schedule(opts.sync_type, opts.ctas_per_sm, opts.cta_threads) != GDP_OKAY) return GDP_ERROR;
    stamps.mark(5);
    GDP_CUDA(cudaStreamSynchronize(ups.s));
    GDP_CUDA(cudaStreamSynchronize(stream));  // before the raw CSR is freed and the verdict is read
    stamps.mark(6);
    stamps.report();
    raw.release();
    return element_error(hbad);
}

// Grid sizes of the loop drivers for the schedule (the layout is untouched).
GDP_RETCODE Context::set_schedule(int sync_type, int ctas_per_sm, int cta_threads) {
    if (sync_type < CPU_LOOP || sync_type > MEGAKERNEL) {
        set_error("Unknown sync type");
        return GDP_ERROR;
    }
    if (cta_threads != 128 && cta_threads != 256 && cta_threads != 512) {
        set_error("cta_threads must be 128, 256 or 512");
        return GDP_ERROR;
    }
    GDP_CUDA(cudaSetDevice(opts.device));
    const int warps = cta_threads / 32;
    int act_bps = 0, cand_bps = 0, mega_bps = 0;
    GDP_CUDA(phase_occupancy(&act_bps, &cand_bps, &mega_bps, warps));
    if (ctas_per_sm > 0) {
        act_bps = std::min(act_bps, ctas_per_sm);
        cand_bps = std::min(cand_bps, ctas_per_sm);
        mega_bps = std::min(mega_bps, ctas_per_sm);
    }
    act_blocks = std::max(1, std::min(act_bps * n_sms, (P.n_items + kWarpsPerCta - 1) / kWarpsPerCta));
    cand_blocks = std::max(1, cand_bps * n_sms);  // the exact-rows phase shares this launch
    mega_grid = std::max(1, mega_bps) * n_sms;
    mega_warps = warps;
    if (graph_exec && (opts.ctas_per_sm != ctas_per_sm)) {  // the GPU_LOOP graph holds the old grids
        cudaGraphExecDestroy(graph_exec);
        cudaGraphDestroy(graph);
        graph_exec = nullptr;
        graph = nullptr;
    }
    opts.sync_type = sync_type;
    opts.ctas_per_sm = ctas_per_sm;
    opts.cta_threads = cta_threads;
    return GDP_OKAY;
}

Context::~Context() {
    if (stream) cudaStreamSynchronize(stream);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (h_flags) cudaFreeHost(h_flags);
    if (stream) cudaStreamDestroy(stream);
}

// ---- drivers ---------------------------------------------------------------
// CPU_LOOP: the host launches each round's phases and reads the flags.
GDP_RETCODE Context::rounds_cpu_loop(cudaStream_t s, int *launches) {
    GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
    GDP_CUDA(cudaStreamSynchronize(s));
    bool go = !h_flags[0].infeasible;
    for (int r = 1; go && r <= opts.max_rounds; r++) {
        GDP_CUDA(launch_round_begin(P, s));
        GDP_CUDA(launch_activity_phase(P, act_blocks, s));
        GDP_CUDA(launch_candidate_phase(P, cand_blocks, s));
        GDP_CUDA(launch_exact_phase(P, cand_blocks, s));
        GDP_CUDA(launch_finalize(P, vec_blocks, s));
        *launches += 2 + (P.n_items > 0) + (P.n_mtiles > 0 || P.defer_exact) + (P.n_mtiles > 0);
        GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
        GDP_CUDA(cudaStreamSynchronize(s));
        go = h_flags[0].change && !h_flags[0].infeasible;
    }
    return GDP_OKAY;
}

// GPU_LOOP: one CUDA graph whose conditional WHILE node repeats the round's
// phase kernels until the condition kernel clears it -- the device-driven loop
// the reference built with dynamic parallelism (src/kernels/atomic_kernel.cuh:452-503).
GDP_RETCODE Context::build_graph(cudaStream_t s) {
    cudaGraph_t g = nullptr;
    GDP_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    GDP_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault));
    // cudaGraphNodeParams has no usable default constructor in C++: zero a raw buffer
    alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
    std::memset(cp_buf, 0, sizeof(cp_buf));
    cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(cp_buf);
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    GDP_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t cs;
    GDP_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    GDP_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    int rc = launch_round_begin(P, cs);
    if (!rc) rc = launch_activity_phase(P, act_blocks, cs);
    if (!rc) rc = launch_candidate_phase(P, cand_blocks, cs);
    if (!rc) rc = launch_exact_phase(P, cand_blocks, cs);
    if (!rc) rc = launch_finalize(P, vec_blocks, cs);
    if (!rc) rc = launch_condition(P, (unsigned long long)h, cs);
    cudaGraph_t captured = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(cs, &captured);
    cudaStreamDestroy(cs);
    (void)s;
    if (rc || ec != cudaSuccess) {
        cudaGraphDestroy(g);
        set_error(std::string("GPU_LOOP graph capture failed: ") +
                  cudaGetErrorString(rc ? (cudaError_t)rc : ec));
        return GDP_ERROR;
    }
    cudaGraphExec_t ge = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&ge, g, 0);
    if (ei != cudaSuccess) {
        cudaGraphDestroy(g);
        set_error(std::string("GPU_LOOP graph instantiation failed: ") + cudaGetErrorString(ei));
        return GDP_ERROR;
    }
    graph = g;
    graph_exec = ge;
    return GDP_OKAY;
}

GDP_RETCODE Context::rounds_gpu_loop(cudaStream_t s, int *launches) {
    if (!graph_exec && build_graph(s) != GDP_OKAY) return GDP_ERROR;
    GDP_CUDA(cudaGraphLaunch(graph_exec, s));
    GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
    GDP_CUDA(cudaStreamSynchronize(s));
    *launches += h_flags[0].rounds * (3 + (P.n_items > 0) + (P.n_mtiles > 0 || P.defer_exact) + (P.n_mtiles > 0)) + 1;
    return GDP_OKAY;
}

// MEGAKERNEL: every round in one persistent cooperative launch.
GDP_RETCODE Context::rounds_megakernel(cudaStream_t s, int *launches) {
    GDP_CUDA(launch_megakernel(P, mega_grid, mega_warps, s));
    *launches += 1;
    GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
    GDP_CUDA(cudaStreamSynchronize(s));
    return GDP_OKAY;
}

GDP_RETCODE Context::run(const double *lb_in, const double *ub_in, double *lb_out, double *ub_out,
                         cudaStream_t s, gdp_stats *st) {
    P.max_rounds = opts.max_rounds;
    certified = false;
    RoundFlags init[3];
    std::memset(init, 0, sizeof(init));
    init[0].infeasible_var = INT_MAX;
    init[0].infeasible_row = INT_MAX;
    GDP_CUDA(cudaMemcpyAsync(P.flags, init, sizeof(init), cudaMemcpyHostToDevice, s));
    GDP_CUDA(cudaMemsetAsync(P.queue, 0, sizeof(unsigned) * 8, s));
    GDP_CUDA(cudaMemsetAsync(P.xctr, 0, sizeof(unsigned) * 32, s));
    GDP_CUDA(cudaMemsetAsync(P.row_exact, 0, sizeof(int) * (size_t)std::max(P.n_lrows, 1), s));
    GDP_CUDA(cudaMemsetAsync(P.barrier, 0, sizeof(unsigned) * 2, s));
    GDP_CUDA(cudaMemsetAsync(P.chg, 0, sizeof(unsigned) * (size_t)std::max(P.n_chg_words, 1), s));
    GDP_CUDA(launch_interleave(P, lb_in, ub_in, vec_blocks, s));
    GDP_CUDA(launch_mark_all(P, vec_blocks, s));  // clear round stamps of earlier propagations
    GDP_CUDA(launch_check_bounds(P, vec_blocks, s));
    int launches = 3;
    GDP_CUDA(cudaEventRecord(ev0, s));
    GDP_RETCODE rc;
    if (P.learned) rc = rounds_learned(s, &launches);
    else if (opts.sync_type == MEGAKERNEL) rc = rounds_megakernel(s, &launches);
    else if (opts.sync_type == GPU_LOOP) rc = rounds_gpu_loop(s, &launches);
    else rc = rounds_cpu_loop(s, &launches);
    if (rc != GDP_OKAY) return rc;
    GDP_CUDA(cudaEventRecord(ev1, s));
    GDP_CUDA(launch_deinterleave(P, lb_out, ub_out, vec_blocks, s));
    launches++;
    GDP_CUDA(cudaStreamSynchronize(s));
    const RoundFlags &f = h_flags[0];
    if (f.error != kErrNone) {
        set_error("device error " + std::to_string(f.error) + " (grid barrier wait exceeded its limit)");
        if (st) st->device_error = f.error;
        return GDP_ERROR;
    }
    // P.bnd now holds a fixpoint certified by a round that changed nothing
    certified = !f.infeasible && !f.change;
    if (st) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess) {
            ms = -1.f;
            cudaGetLastError();
        }
        st->rounds = f.rounds;
        st->infeasible = f.infeasible;
        st->infeasible_var = (f.infeasible && f.infeasible_var != INT_MAX) ? f.infeasible_var : -1;
        st->infeasible_row = (f.infeasible && f.infeasible_row != INT_MAX) ? f.infeasible_row : -1;
        st->converged = (f.infeasible || !f.change) ? 1 : 0;
        st->device_error = f.error;
        st->kernel_launches = launches;
        st->changed_vars = (long long)f.changed_vars;
        st->rows_processed = (long long)f.rows_proc;
        st->nnz_processed = (long long)f.nnz_proc;
        st->nnz_exact = (long long)f.nnz_exact;
        st->rows_deferred = (long long)f.rows_deferred;
        st->divisions = (long long)f.divisions;
        st->rows_exact = (long long)f.rows_exact;
        st->rows_go = (long long)f.rows_go;
        st->rows_seqmax = (long long)f.rows_seqmax;
        st->rows_drift = (long long)f.rows_drift;
        st->nnz_drift = (long long)f.nnz_drift;
        st->full_rounds = f.full_rounds;
        // the rows read: without those left unread on their drift bound
        st->bytes_algorithmic = 12.0 * (double)(f.nnz_proc - f.nnz_drift) + 20.0 * (double)(f.rows_proc - f.rows_drift) +
                                36.0 * n * (double)f.rounds;
        st->device_ms = ms;
    }
    return GDP_OKAY;
}

// Learned marking: every round in one launch of the learned round loop.
GDP_RETCODE Context::rounds_learned(cudaStream_t s, int *launches) {
    DevProblem Q = P;
    Q.defer_exact = 0;  // labels and row state need each row's outcome in its own warp
    GDP_CUDA((cudaError_t)launch_learned(Q, learned_grid, vec_blocks, s));
    *launches += 2;
    GDP_CUDA(cudaMemcpyAsync(h_flags, P.flags, sizeof(RoundFlags), cudaMemcpyDeviceToHost, s));
    GDP_CUDA(cudaStreamSynchronize(s));
    return GDP_OKAY;
}

GDP_RETCODE Context::alloc_learned_state() {
    if (P.dirty) return GDP_OKAY;
    const size_t ns = (size_t)std::max(P.n_srows, 1);
    P.dirty = (int *)arena.alloc_bytes(sizeof(int) * ns);
    P.dcount = (int *)arena.alloc_bytes(sizeof(int) * ns);
    P.last_proc = (int *)arena.alloc_bytes(sizeof(int) * ns);
    P.last_tight = (int *)arena.alloc_bytes(sizeof(int) * ns);
    P.rstat = (float2 *)arena.alloc_bytes(sizeof(float2) * ns);
    P.rinfo = (unsigned *)arena.alloc_bytes(sizeof(unsigned) * ns);
    P.trace_n = (unsigned *)arena.alloc_bytes(sizeof(unsigned));
    if (!P.dirty || !P.dcount || !P.last_proc || !P.last_tight || !P.rstat || !P.rinfo || !P.trace_n) {
        set_error("device allocation failed (learned marking state)");
        return GDP_ERROR;
    }
    int bps = 0;
    GDP_CUDA((cudaError_t)learned_occupancy(&bps));
    learned_grid = std::max(1, bps) * n_sms;
    return GDP_OKAY;
}

GDP_RETCODE Context::set_model(const Mlp *m, float threshold, int min_len) {
    if (!m) {
        P.learned = 0;
        return GDP_OKAY;
    }
    if (alloc_learned_state() != GDP_OKAY) return GDP_ERROR;
    P.mlp = m->dev();
    P.tau = threshold;
    P.learn_min_len = std::max(0, min_len);
    P.learned = 1;
    return GDP_OKAY;
}

GDP_RETCODE Context::trace(double *lbs, double *ubs, int capacity, float *x_out, float *y_out, int *n_out,
                           gdp_stats *st) {
    if (capacity < 0 || (capacity > 0 && (!x_out || !y_out)) || !n_out) {
        set_error("bad trace arguments");
        return GDP_ERROR;
    }
    if (alloc_learned_state() != GDP_OKAY) return GDP_ERROR;
    const size_t cap = (size_t)std::max(capacity, 1);
    float *dx = nullptr, *dy = nullptr;
    GDP_CUDA(cudaMalloc(&dx, sizeof(float) * 16 * cap));
    GDP_CUDA(cudaMalloc(&dy, sizeof(float) * cap));
    const int saved = P.learned;
    P.learned = 2;
    P.trace_x = dx;
    P.trace_y = dy;
    P.trace_cap = (unsigned)capacity;
    GDP_RETCODE rc = GDP_OKAY;
    if (cudaMemsetAsync(P.trace_n, 0, sizeof(unsigned), stream) != cudaSuccess) rc = GDP_ERROR;
    if (rc == GDP_OKAY) rc = propagate_host(lbs, ubs, st);
    P.learned = saved;
    P.trace_x = nullptr;
    P.trace_y = nullptr;
    P.trace_cap = 0;
    unsigned cnt = 0;
    if (rc == GDP_OKAY) {
        if (cudaMemcpy(&cnt, P.trace_n, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) rc = GDP_ERROR;
        const unsigned keep = std::min(cnt, (unsigned)capacity);
        if (rc == GDP_OKAY && keep) {
            if (cudaMemcpy(x_out, dx, sizeof(float) * 16 * keep, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(y_out, dy, sizeof(float) * keep, cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = GDP_ERROR;
        }
        *n_out = (int)keep;
        if (rc != GDP_OKAY) set_error("trace download failed");
    }
    cudaFree(dx);
    cudaFree(dy);
    return rc;
}

GDP_RETCODE Context::propagate_host(double *lbs, double *ubs, gdp_stats *st) {
    if (host_direct) {
        // coherent access to pageable memory (NVLink-C2C on Grace hosts): the
        // first kernel reads the caller's bounds where they are, and the
        // result is written back to them by a kernel once the run succeeded
        if (run(lbs, ubs, d_lb, d_ub, stream, st) != GDP_OKAY) return GDP_ERROR;
        GDP_CUDA(launch_copy_out(d_lb, d_ub, lbs, ubs, n, vec_blocks, stream));
        GDP_CUDA(cudaStreamSynchronize(stream));
        return GDP_OKAY;
    }
    const size_t bytes = sizeof(double) * (size_t)n;
    GDP_CUDA(cudaMemcpyAsync(d_lb, lbs, bytes, cudaMemcpyHostToDevice, stream));
    GDP_CUDA(cudaMemcpyAsync(d_ub, ubs, bytes, cudaMemcpyHostToDevice, stream));
    if (run(d_lb, d_ub, d_lb, d_ub, stream, st) != GDP_OKAY) return GDP_ERROR;
    GDP_CUDA(cudaMemcpyAsync(lbs, d_lb, bytes, cudaMemcpyDeviceToHost, stream));
    GDP_CUDA(cudaMemcpyAsync(ubs, d_ub, bytes, cudaMemcpyDeviceToHost, stream));
    GDP_CUDA(cudaStreamSynchronize(stream));
    return GDP_OKAY;
}

GDP_RETCODE Context::propagate_device(double *d_lbs, double *d_ubs, cudaStream_t s, gdp_stats *st) {
    if (!s) s = stream;
    return run(d_lbs, d_ubs, d_lbs, d_ubs, s, st);
}

}  // namespace gdp

// gdp_mlp.cu -- training and inference kernels of the row-marking MLP
// (16 -> 64 -> 64 -> 1, ReLU, BF16 weights/activations, FP32 accumulation)
// and its C-ABI (gdp_mlp_*).
//
// Training minimises the weighted binary cross-entropy of sigmoid(z) against
// the label "processing this row tightened a bound" with Adam on FP32 master
// weights; BF16 copies are refreshed after every step.
//
// Backward of one 16-sample tile (one warp), in the forward's fragment layout:
//   dz      = w (sigmoid(z) - y) / sum(w)
//   g_w3   += dz relu(a2),            g_b3 += dz
//   da2     = dz w3 [a2 > 0]          (FP32)
//   g_W2   += da2^T bf16(relu(a1)),   g_b2 += da2        (FP32, CUDA cores)
//   dh1     = bf16(da2) @ W2          (tensor cores, W2^T as the B operand)
//   da1     = dh1 [a1 > 0]
//   g_W1   += da1^T x,                g_b1 += da1        (FP32, CUDA cores)
// Weight gradients of a CTA accumulate in shared memory and reach global
// memory with one atomic per parameter per CTA.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gdp_context.h"
#include "gdp_mlp.h"

namespace gdp {

namespace {

constexpr int kMlpWarps = 4;
constexpr int kMlpThreads = 32 * kMlpWarps;

// Per-warp tile scratch (FP32): da2, h1 (bf16-rounded relu(a1)), da1, x.
// Rows of 64 values are padded to 72 floats: the fragment-layout stores and
// loads (lanes 4g + t at row g, column 2t + c) then meet at most 2 lanes per
// bank instead of 8.
constexpr int kTileLd = kMlpH + 8;
struct TileSmem {
    float da2[16][kTileLd];
    float h1[16][kTileLd];
    float da1[16][kTileLd];
    float x[16][kMlpIn];
};

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// A registers of rows [r0, r0 + 16) of a row-major BF16 [n][16] array (zero past n).
__device__ __forceinline__ void load_a_global(const __nv_bfloat16 *X, int n, int r0, int lane, unsigned (&a)[4]) {
    const int g = lane >> 2, t = lane & 3;
    const int ra = r0 + g, rb = r0 + g + 8;
    a[0] = ra < n ? __ldg(reinterpret_cast<const unsigned *>(X + (size_t)ra * 16 + 2 * t)) : 0u;
    a[1] = rb < n ? __ldg(reinterpret_cast<const unsigned *>(X + (size_t)rb * 16 + 2 * t)) : 0u;
    a[2] = ra < n ? __ldg(reinterpret_cast<const unsigned *>(X + (size_t)ra * 16 + 2 * t + 8)) : 0u;
    a[3] = rb < n ? __ldg(reinterpret_cast<const unsigned *>(X + (size_t)rb * 16 + 2 * t + 8)) : 0u;
}

__global__ void __launch_bounds__(kMlpThreads) k_mlp_forward(MlpDev M, const __nv_bfloat16 *X, int n, float *z) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int r0 = warp * 16; r0 < n; r0 += nwarps * 16) {
        unsigned a[4];
        load_a_global(X, n, r0, lane, a);
        MlpTile T;
        mlp_forward_tile(M, a, lane, T);
        const int g = lane >> 2;
        if ((lane & 3) == 0) {
            if (r0 + g < n) z[r0 + g] = T.z[0];
            if (r0 + g + 8 < n) z[r0 + g + 8] = T.z[1];
        }
    }
}

// Gradient of the weighted BCE over samples [0, n); grad (kMlpParams floats,
// zeroed by the caller) and loss (1 float) receive atomic adds.
__global__ void __launch_bounds__(kMlpThreads) k_mlp_grad(MlpDev M, const __nv_bfloat16 *X, const float *y,
                                                           const float *w, int n, float inv_wsum, float *grad,
                                                           float *loss) {
    extern __shared__ float4 smem_raw[];
    float *acc = reinterpret_cast<float *>(smem_raw);  // kMlpParams
    TileSmem *tiles = reinterpret_cast<TileSmem *>(acc + ((kMlpParams + 3) & ~3));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    TileSmem &S = tiles[wid];
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    float *gW1 = acc + kOffW1, *gb1 = acc + kOffB1, *gW2 = acc + kOffW2, *gb2 = acc + kOffB2, *gw3 = acc + kOffW3,
          *gb3 = acc + kOffB3;
    const int g = lane >> 2, t = lane & 3;
    const int warp = blockIdx.x * kMlpWarps + wid, nwarps = gridDim.x * kMlpWarps;
    float lsum = 0.f;
    for (int r0 = warp * 16; r0 < n; r0 += nwarps * 16) {
        unsigned a[4];
        load_a_global(X, n, r0, lane, a);
        MlpTile T;
        mlp_forward_tile(M, a, lane, T);
        // per-row dz (rows g and g + 8)
        float dz[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int r = r0 + g + 8 * h;
            dz[h] = 0.f;
            if (r < n) {
                const float zz = T.z[h], yy = __ldg(y + r), ww = __ldg(w + r);
                const float p = 1.f / (1.f + __expf(-zz));
                dz[h] = ww * (p - yy) * inv_wsum;
                // BCE with logits: max(z, 0) - z y + log(1 + exp(-|z|))
                if (t == 0) lsum += ww * (fmaxf(zz, 0.f) - zz * yy + log1pf(__expf(-fabsf(zz)))) * inv_wsum;
            }
        }
        // layer 3 and da2
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
#pragma unroll
            for (int c = 0; c < 2; c++) {
                const int col = nt * 8 + 2 * t + c;
                const float w3 = __bfloat162float(M.w3[col]);
                const float h0 = fmaxf(T.a2[nt][c], 0.f), h8 = fmaxf(T.a2[nt][2 + c], 0.f);
                float gw = dz[0] * h0 + dz[1] * h8;
                gw += __shfl_xor_sync(0xffffffffu, gw, 4);
                gw += __shfl_xor_sync(0xffffffffu, gw, 8);
                gw += __shfl_xor_sync(0xffffffffu, gw, 16);
                if (g == 0) atomicAdd(gw3 + col, gw);
                S.da2[g][col] = T.a2[nt][c] > 0.f ? dz[0] * w3 : 0.f;
                S.da2[g + 8][col] = T.a2[nt][2 + c] > 0.f ? dz[1] * w3 : 0.f;
                S.h1[g][col] = bf16r(fmaxf(T.a1[nt][c], 0.f));
                S.h1[g + 8][col] = bf16r(fmaxf(T.a1[nt][2 + c], 0.f));
            }
        }
        {
            float gb = (t == 0) ? dz[0] + dz[1] : 0.f;
            for (int off = 16; off > 0; off >>= 1) gb += __shfl_xor_sync(0xffffffffu, gb, off);
            if (lane == 0) atomicAdd(gb3, gb);
        }
        // x tile (FP32 copy of the BF16 inputs)
        for (int i = lane; i < 16 * kMlpIn; i += 32) {
            const int r = i / kMlpIn, k = i % kMlpIn;
            S.x[r][k] = r0 + r < n ? __bfloat162float(X[(size_t)(r0 + r) * kMlpIn + k]) : 0.f;
        }
        __syncwarp();
        // dh1 = bf16(da2) @ W2 on the tensor cores
        unsigned da[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            da[kt][0] = pack_bf16(S.da2[g][kt * 16 + 2 * t], S.da2[g][kt * 16 + 2 * t + 1]);
            da[kt][1] = pack_bf16(S.da2[g + 8][kt * 16 + 2 * t], S.da2[g + 8][kt * 16 + 2 * t + 1]);
            da[kt][2] = pack_bf16(S.da2[g][kt * 16 + 2 * t + 8], S.da2[g][kt * 16 + 2 * t + 9]);
            da[kt][3] = pack_bf16(S.da2[g + 8][kt * 16 + 2 * t + 8], S.da2[g + 8][kt * 16 + 2 * t + 9]);
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
                unsigned b0, b1;
                load_bfrag(M.w2t, 4, nt, kt, lane, b0, b1);
                mma_bf16(c, da[kt], b0, b1);
            }
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const int col = nt * 8 + 2 * t + cc;
                S.da1[g][col] = T.a1[nt][cc] > 0.f ? c[cc] : 0.f;
                S.da1[g + 8][col] = T.a1[nt][2 + cc] > 0.f ? c[2 + cc] : 0.f;
            }
        }
        __syncwarp();
        // weight gradients of the tile, each a sum over its 16 samples in
        // sample order. Lanes own columns: a row's reads are broadcasts and
        // the 32 shared-memory adds of one instruction go to 32 banks.
        //   b2, b1: lane owns rows lane and lane + 32
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int row = lane + 32 * q;
            float sb2 = 0.f, sb1 = 0.f;
            for (int s = 0; s < 16; s++) {
                sb2 += S.da2[s][row];
                sb1 += S.da1[s][row];
            }
            atomicAdd(gb2 + row, sb2);
            atomicAdd(gb1 + row, sb1);
        }
        {  // W2: lane owns columns lane and lane + 32 of every row
            float hl[16], hh[16];
#pragma unroll
            for (int s = 0; s < 16; s++) {
                hl[s] = S.h1[s][lane];
                hh[s] = S.h1[s][lane + 32];
            }
            for (int row = 0; row < kMlpH; row++) {
                float vl = 0.f, vh = 0.f;
#pragma unroll
                for (int s = 0; s < 16; s++) {
                    const float d = S.da2[s][row];
                    vl = fmaf(d, hl[s], vl);
                    vh = fmaf(d, hh[s], vh);
                }
                atomicAdd(gW2 + row * kMlpH + lane, vl);
                atomicAdd(gW2 + row * kMlpH + lane + 32, vh);
            }
        }
        {  // W1: lane owns column lane & 15 of the rows of parity lane >> 4
            const int k = lane & 15;
            float xs[16];
#pragma unroll
            for (int s = 0; s < 16; s++) xs[s] = S.x[s][k];
            for (int rr = 0; rr < kMlpH / 2; rr++) {
                const int row = 2 * rr + (lane >> 4);
                float v = 0.f;
#pragma unroll
                for (int s = 0; s < 16; s++) v = fmaf(S.da1[s][row], xs[s], v);
                atomicAdd(gW1 + row * kMlpIn + k, v);
            }
        }
        __syncwarp();
    }
    for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    if (lane == 0) atomicAdd(loss, lsum);
    __syncthreads();
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x)
        if (acc[i] != 0.f) atomicAdd(grad + i, acc[i]);
}

// Adam step on the FP32 master parameters, then the BF16 copies.
__global__ void k_mlp_adam(float *p, float *m1, float *m2, const float *grad, int step, float lr, float beta1,
                           float beta2, float eps) {
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParams; i += gridDim.x * blockDim.x) {
        const float gr = grad[i];
        const float a = beta1 * m1[i] + (1.f - beta1) * gr;
        const float b = beta2 * m2[i] + (1.f - beta2) * gr * gr;
        m1[i] = a;
        m2[i] = b;
        p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
    }
}

// BF16 copies of the master weights, W1, W2 and W2 transposed in fragment
// order (frag_index).
__global__ void k_mlp_cast(const float *p, __nv_bfloat16 *w1, __nv_bfloat16 *w2, __nv_bfloat16 *w2t,
                           __nv_bfloat16 *w3) {
    static_assert(kMlpIn == 16 && kMlpH % 16 == 0, "one k-tile for layer 1, whole k-tiles for layer 2");
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpH * kMlpH; i += gridDim.x * blockDim.x) {
        const int r = i / kMlpH, c = i % kMlpH;
        const __nv_bfloat16 v = __float2bfloat16_rn(p[kOffW2 + i]);
        w2[frag_index(r, c, kMlpH / 16)] = v;
        w2t[frag_index(c, r, kMlpH / 16)] = v;
        if (i < kMlpH * kMlpIn) w1[frag_index(i / kMlpIn, i % kMlpIn, 1)] = __float2bfloat16_rn(p[kOffW1 + i]);
        if (i < kMlpH) w3[i] = __float2bfloat16_rn(p[kOffW3 + i]);
    }
}

__global__ void k_to_bf16(const float *x, __nv_bfloat16 *y, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}

}  // namespace

// ---- host ---------------------------------------------------------------------
#define GDP_MCUDA(call)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call);      \
            return GDP_ERROR;                                                                    \
        }                                                                                        \
    } while (0)

namespace {
constexpr size_t kGradSmem = sizeof(float) * ((kMlpParams + 3) & ~3) + sizeof(TileSmem) * kMlpWarps;

unsigned long long splitmix(unsigned long long &s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
double uniform01(unsigned long long &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

int device_sms() {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// Gradient: two CTAs per SM (its registers allow no more), at most one per 4 tiles.
int grad_grid(int n) {
    const int tiles = (n + 15) / 16;
    return std::max(1, std::min(2 * device_sms(), (tiles + kMlpWarps - 1) / kMlpWarps));
}

// Forward: every CTA that fits on an SM (the loop waits on its loads, and more
// warps hide them), at most one per 4 tiles.
int forward_grid(int n) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlp_forward, kMlpThreads, 0) != cudaSuccess ||
        per_sm < 1)
        per_sm = 2;
    const int tiles = (n + 15) / 16;
    return std::max(1, std::min(per_sm * device_sms(), (tiles + kMlpWarps - 1) / kMlpWarps));
}
}  // namespace

Mlp::~Mlp() {
    if (stream) cudaStreamSynchronize(stream);
    for (void *q : {(void *)p, (void *)m1, (void *)m2, (void *)grad, (void *)loss, (void *)w1, (void *)w2,
                    (void *)w2t, (void *)w3})
        if (q) cudaFree(q);
    if (stream) cudaStreamDestroy(stream);
}

MlpDev Mlp::dev() const {
    MlpDev d;
    d.w1 = w1; d.w2 = w2; d.w2t = w2t; d.w3 = w3;
    d.b1 = p + kOffB1; d.b2 = p + kOffB2; d.b3 = p + kOffB3;
    return d;
}

GDP_RETCODE Mlp::refresh_bf16() {
    k_mlp_cast<<<16, 256, 0, stream>>>(p, w1, w2, w2t, w3);
    GDP_MCUDA(cudaGetLastError());
    return GDP_OKAY;
}

GDP_RETCODE Mlp::init(unsigned long long seed, int dev_index) {
    device = dev_index;
    GDP_MCUDA(cudaSetDevice(device));
    GDP_MCUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    const size_t pb = sizeof(float) * kMlpParams;
    GDP_MCUDA(cudaMalloc(&p, pb));
    GDP_MCUDA(cudaMalloc(&m1, pb));
    GDP_MCUDA(cudaMalloc(&m2, pb));
    GDP_MCUDA(cudaMalloc(&grad, pb));
    GDP_MCUDA(cudaMalloc(&loss, sizeof(float)));
    GDP_MCUDA(cudaMalloc(&w1, sizeof(__nv_bfloat16) * kMlpH * kMlpIn));
    GDP_MCUDA(cudaMalloc(&w2, sizeof(__nv_bfloat16) * kMlpH * kMlpH));
    GDP_MCUDA(cudaMalloc(&w2t, sizeof(__nv_bfloat16) * kMlpH * kMlpH));
    GDP_MCUDA(cudaMalloc(&w3, sizeof(__nv_bfloat16) * kMlpH));
    GDP_MCUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem));
    // He-uniform weights, zero biases
    std::vector<float> h(kMlpParams, 0.f);
    unsigned long long s = seed;
    auto fill = [&](int off, int count, int fan_in) {
        const double a = std::sqrt(6.0 / fan_in);
        for (int i = 0; i < count; i++) h[off + i] = (float)((2.0 * uniform01(s) - 1.0) * a);
    };
    fill(kOffW1, kMlpH * kMlpIn, kMlpIn);
    fill(kOffW2, kMlpH * kMlpH, kMlpH);
    fill(kOffW3, kMlpH, kMlpH);
    return set(h.data());
}

GDP_RETCODE Mlp::set(const float *params) {
    if (!params) { set_error("null parameters"); return GDP_ERROR; }
    GDP_MCUDA(cudaMemcpyAsync(p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, stream));
    GDP_MCUDA(cudaMemsetAsync(m1, 0, sizeof(float) * kMlpParams, stream));
    GDP_MCUDA(cudaMemsetAsync(m2, 0, sizeof(float) * kMlpParams, stream));
    step = 0;
    if (refresh_bf16() != GDP_OKAY) return GDP_ERROR;
    GDP_MCUDA(cudaStreamSynchronize(stream));
    return GDP_OKAY;
}

GDP_RETCODE Mlp::get(float *params) const {
    if (!params) { set_error("null parameters"); return GDP_ERROR; }
    GDP_MCUDA(cudaMemcpyAsync(params, p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream));
    GDP_MCUDA(cudaStreamSynchronize(stream));
    return GDP_OKAY;
}

namespace {
// Uploads n x 16 FP32 features as BF16 (device buffer owned by the caller).
GDP_RETCODE upload_x(const float *x, int n, __nv_bfloat16 **out, cudaStream_t s) {
    float *tmp = nullptr;
    const size_t cnt = (size_t)n * kMlpIn;
    GDP_MCUDA(cudaMalloc(&tmp, sizeof(float) * std::max<size_t>(cnt, 1)));
    GDP_MCUDA(cudaMalloc(out, sizeof(__nv_bfloat16) * std::max<size_t>(cnt, 1)));
    if (cnt) {
        GDP_MCUDA(cudaMemcpyAsync(tmp, x, sizeof(float) * cnt, cudaMemcpyHostToDevice, s));
        k_to_bf16<<<256, 256, 0, s>>>(tmp, *out, (long long)cnt);
        GDP_MCUDA(cudaGetLastError());
    }
    GDP_MCUDA(cudaStreamSynchronize(s));
    cudaFree(tmp);
    return GDP_OKAY;
}
}  // namespace

GDP_RETCODE Mlp::forward(int n, const float *x, float *z) {
    if (n < 0 || (n && (!x || !z))) { set_error("bad forward arguments"); return GDP_ERROR; }
    if (!n) return GDP_OKAY;
    __nv_bfloat16 *xb = nullptr;
    float *dz = nullptr;
    if (upload_x(x, n, &xb, stream) != GDP_OKAY) return GDP_ERROR;
    GDP_MCUDA(cudaMalloc(&dz, sizeof(float) * n));
    k_mlp_forward<<<forward_grid(n), kMlpThreads, 0, stream>>>(dev(), xb, n, dz);
    GDP_MCUDA(cudaGetLastError());
    GDP_MCUDA(cudaMemcpyAsync(z, dz, sizeof(float) * n, cudaMemcpyDeviceToHost, stream));
    GDP_MCUDA(cudaStreamSynchronize(stream));
    cudaFree(xb);
    cudaFree(dz);
    return GDP_OKAY;
}

GDP_RETCODE Mlp::gradient(int n, const float *x, const float *y, const float *w, float *g, float *lossv) {
    if (n <= 0 || !x || !y || !w || !g) { set_error("bad gradient arguments"); return GDP_ERROR; }
    __nv_bfloat16 *xb = nullptr;
    float *dy = nullptr, *dw = nullptr;
    if (upload_x(x, n, &xb, stream) != GDP_OKAY) return GDP_ERROR;
    GDP_MCUDA(cudaMalloc(&dy, sizeof(float) * n));
    GDP_MCUDA(cudaMalloc(&dw, sizeof(float) * n));
    GDP_MCUDA(cudaMemcpyAsync(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice, stream));
    GDP_MCUDA(cudaMemcpyAsync(dw, w, sizeof(float) * n, cudaMemcpyHostToDevice, stream));
    double ws = 0.0;
    for (int i = 0; i < n; i++) ws += w[i];
    GDP_MCUDA(cudaMemsetAsync(grad, 0, sizeof(float) * kMlpParams, stream));
    GDP_MCUDA(cudaMemsetAsync(loss, 0, sizeof(float), stream));
    k_mlp_grad<<<grad_grid(n), kMlpThreads, kGradSmem, stream>>>(dev(), xb, dy, dw, n,
                                                                   ws > 0 ? (float)(1.0 / ws) : 0.f, grad, loss);
    GDP_MCUDA(cudaGetLastError());
    GDP_MCUDA(cudaMemcpyAsync(g, grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream));
    float l = 0.f;
    GDP_MCUDA(cudaMemcpyAsync(&l, loss, sizeof(float), cudaMemcpyDeviceToHost, stream));
    GDP_MCUDA(cudaStreamSynchronize(stream));
    if (lossv) *lossv = l;
    cudaFree(xb);
    cudaFree(dy);
    cudaFree(dw);
    return GDP_OKAY;
}

GDP_RETCODE Mlp::train(int n, const float *x, const float *y, const float *w, int epochs, int batch, float lr,
                       unsigned long long seed, float *final_loss) {
    if (n <= 0 || !x || !y || !w || epochs <= 0 || batch <= 0 || !(lr > 0.f)) {
        set_error("bad training arguments");
        return GDP_ERROR;
    }
    // one shuffle of the samples; epochs walk contiguous minibatches from a
    // rotating start
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    unsigned long long s = seed;
    for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[(int)(splitmix(s) % (unsigned long long)(i + 1))]);
    std::vector<float> xs((size_t)n * kMlpIn), ys(n), wsv(n);
    std::vector<double> wpre(n + 1, 0.0);
    for (int i = 0; i < n; i++) {
        const int k = perm[i];
        std::memcpy(&xs[(size_t)i * kMlpIn], x + (size_t)k * kMlpIn, sizeof(float) * kMlpIn);
        ys[i] = y[k];
        wsv[i] = w[k];
        wpre[i + 1] = wpre[i] + w[k];
    }
    __nv_bfloat16 *xb = nullptr;
    float *dy = nullptr, *dw = nullptr;
    if (upload_x(xs.data(), n, &xb, stream) != GDP_OKAY) return GDP_ERROR;
    GDP_MCUDA(cudaMalloc(&dy, sizeof(float) * n));
    GDP_MCUDA(cudaMalloc(&dw, sizeof(float) * n));
    GDP_MCUDA(cudaMemcpyAsync(dy, ys.data(), sizeof(float) * n, cudaMemcpyHostToDevice, stream));
    GDP_MCUDA(cudaMemcpyAsync(dw, wsv.data(), sizeof(float) * n, cudaMemcpyHostToDevice, stream));
    const int nb = (n + batch - 1) / batch;
    double last = 0.0;
    int last_cnt = 0;
    std::vector<float> lh(nb);
    float *d_losses = nullptr;
    GDP_MCUDA(cudaMalloc(&d_losses, sizeof(float) * nb));
    for (int e = 0; e < epochs; e++) {
        GDP_MCUDA(cudaMemsetAsync(d_losses, 0, sizeof(float) * nb, stream));
        const int rot = (int)(splitmix(s) % (unsigned long long)nb);
        for (int b = 0; b < nb; b++) {
            const int bi = (b + rot) % nb;
            const int r0 = bi * batch, cnt = std::min(batch, n - r0);
            const double ws = wpre[r0 + cnt] - wpre[r0];
            GDP_MCUDA(cudaMemsetAsync(grad, 0, sizeof(float) * kMlpParams, stream));
            k_mlp_grad<<<grad_grid(cnt), kMlpThreads, kGradSmem, stream>>>(
                dev(), xb + (size_t)r0 * kMlpIn, dy + r0, dw + r0, cnt, ws > 0 ? (float)(1.0 / ws) : 0.f, grad,
                d_losses + bi);
            step++;
            k_mlp_adam<<<8, 256, 0, stream>>>(p, m1, m2, grad, step, lr, 0.9f, 0.999f, 1e-8f);
            k_mlp_cast<<<16, 256, 0, stream>>>(p, w1, w2, w2t, w3);
            GDP_MCUDA(cudaGetLastError());
        }
        if (e == epochs - 1) {
            GDP_MCUDA(cudaMemcpyAsync(lh.data(), d_losses, sizeof(float) * nb, cudaMemcpyDeviceToHost, stream));
            GDP_MCUDA(cudaStreamSynchronize(stream));
            for (int b = 0; b < nb; b++) {
                const int r0 = b * batch, cnt = std::min(batch, n - r0);
                last += lh[b] * (wpre[r0 + cnt] - wpre[r0]);
                last_cnt++;
            }
        }
    }
    GDP_MCUDA(cudaStreamSynchronize(stream));
    if (final_loss) *final_loss = wpre[n] > 0 ? (float)(last / wpre[n]) : 0.f;
    cudaFree(xb);
    cudaFree(dy);
    cudaFree(dw);
    cudaFree(d_losses);
    return GDP_OKAY;
}

}  // namespace gdp

// ---- C-ABI ----------------------------------------------------------------------

#pragma GCC visibility push(default)
extern "C" {

GDP_RETCODE gdp_mlp_create(unsigned long long seed, int device, gdp_mlp **out) {
    if (!out) { gdp::set_error("null output pointer"); return GDP_ERROR; }
    *out = nullptr;
    gdp_mlp *m = new (std::nothrow) gdp_mlp();
    if (!m) { gdp::set_error("host allocation failed"); return GDP_ERROR; }
    if (m->impl.init(seed, device) != GDP_OKAY) { delete m; return GDP_ERROR; }
    *out = m;
    return GDP_OKAY;
}

GDP_RETCODE gdp_mlp_destroy(gdp_mlp *m) {
    delete m;
    return GDP_OKAY;
}

GDP_RETCODE gdp_mlp_get_params(const gdp_mlp *m, float *params) {
    if (!m) { gdp::set_error("null model"); return GDP_ERROR; }
    return m->impl.get(params);
}

GDP_RETCODE gdp_mlp_set_params(gdp_mlp *m, const float *params) {
    if (!m) { gdp::set_error("null model"); return GDP_ERROR; }
    return m->impl.set(params);
}

GDP_RETCODE gdp_mlp_forward(gdp_mlp *m, int n, const float *x, float *logits) {
    if (!m) { gdp::set_error("null model"); return GDP_ERROR; }
    return m->impl.forward(n, x, logits);
}

GDP_RETCODE gdp_mlp_gradient(gdp_mlp *m, int n, const float *x, const float *y, const float *w, float *grad,
                             float *loss) {
    if (!m) { gdp::set_error("null model"); return GDP_ERROR; }
    return m->impl.gradient(n, x, y, w, grad, loss);
}

GDP_RETCODE gdp_mlp_train(gdp_mlp *m, int n, const float *x, const float *y, const float *w, int epochs, int batch,
                          float lr, unsigned long long seed, float *final_loss) {
    if (!m) { gdp::set_error("null model"); return GDP_ERROR; }
    return m->impl.train(n, x, y, w, epochs, batch, lr, seed, final_loss);
}

}  // extern "C"
#pragma GCC visibility pop

// gdp_mlp.cuh -- the row-marking MLP on the device: 16 -> 64 -> 64 -> 1 with
// ReLU, BF16 weights and activations, FP32 accumulation.
//
// Forward for a tile of 16 rows (one warp): layers 1 and 2 on the tensor cores
// (mma.sync m16n8k16, BF16 x BF16 -> FP32); layer 1's accumulator fragments
// become layer 2's A fragments in registers (after ReLU and rounding to BF16),
// so activations never leave the warp. Layer 3 is a 64-term FP32 dot product
// per row, reduced across the 4 lanes that hold the row.
//
// Fragment layouts (PTX ISA, mma.m16n8k16 with .bf16 inputs; g = lane >> 2,
// t = lane & 3):
//   A (16 x 16, row-major): {A[g][2t..2t+1]}, {A[g+8][2t..]}, {A[g][2t+8..]},
//                           {A[g+8][2t+8..]}  -- four 32-bit registers
//   B (16 x 8, "col"):      {B[2t..2t+1][g]}, {B[2t+8..2t+9][g]}
//   C (16 x 8, FP32):       C[g][2t], C[g][2t+1], C[g+8][2t], C[g+8][2t+1]
// A weight matrix W[n][k] is the "col" B operand of x @ W^T: B registers hold
// two adjacent k of row n. The BF16 copies are stored in fragment order
// (frag_index), so that a warp reads its B registers in one coalesced load.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace gdp {

constexpr int kMlpIn = 16, kMlpH = 64;

// Device view of one model. Master weights are FP32 (training); the forward
// reads the BF16 copies (in fragment order, frag_index).
struct MlpDev {
    const __nv_bfloat16 *w1;   // [64][16]
    const __nv_bfloat16 *w2;   // [64][64]
    const __nv_bfloat16 *w2t;  // [64][64] transposed (backward)
    const __nv_bfloat16 *w3;   // [64]
    const float *b1, *b2, *b3;  // [64], [64], [1]
};

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half)
    return *reinterpret_cast<const unsigned *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Fragment order of a BF16 weight matrix W[n][k] with kts k-tiles of 16: the
// B registers of n-tile nt (rows 8 nt ..) and k-tile kt for lane 4g + t,
// {W[8nt+g][16kt+2t], W[..][16kt+2t+1]} and {W[..][16kt+2t+8], W[..][16kt+2t+9]},
// are the 8-byte word (nt kts + kt) 32 + lane. Returns W[n][k]'s BF16 index.
__host__ __device__ __forceinline__ int frag_index(int n, int k, int kts) {
    const int nt = n >> 3, g = n & 7, kt = k >> 4, kk = k & 15;
    return (((nt * kts + kt) * 32 + 4 * g + ((kk & 7) >> 1)) << 2) + ((kk >> 3) << 1) + (kk & 1);
}

// B operand registers of n-tile nt, k-tile kt of a weight matrix in fragment
// order with kts k-tiles (a warp reads 256 consecutive bytes).
__device__ __forceinline__ void load_bfrag(const __nv_bfloat16 *Wf, int kts, int nt, int kt, int lane, unsigned &b0,
                                           unsigned &b1) {
    const uint2 v = __ldg(reinterpret_cast<const uint2 *>(Wf) + (nt * kts + kt) * 32 + lane);
    b0 = v.x;
    b1 = v.y;
}

// Layer outputs of a 16-row tile in C-fragment layout: acc[n-tile][4].
struct MlpTile {
    float a1[8][4];  // layer-1 pre-activations (16 x 64)
    float a2[8][4];  // layer-2 pre-activations (16 x 64)
    float z[2];      // logits of rows g and g+8 (valid in every lane of the quad)
};

// Forward of the 16 x 16 input tile given as A registers (BF16).
__device__ __forceinline__ void mlp_forward_tile(const MlpDev &M, const unsigned (&x)[4], int lane, MlpTile &T) {
    const int t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const float bl = __ldg(M.b1 + nt * 8 + 2 * t), bh = __ldg(M.b1 + nt * 8 + 2 * t + 1);
        T.a1[nt][0] = bl; T.a1[nt][1] = bh; T.a1[nt][2] = bl; T.a1[nt][3] = bh;
        unsigned b0, b1;
        load_bfrag(M.w1, 1, nt, 0, lane, b0, b1);
        mma_bf16(T.a1[nt], x, b0, b1);
    }
    // layer-1 accumulators -> layer-2 A fragments (ReLU, BF16)
    unsigned h[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        const float *c0 = T.a1[2 * kt], *c1 = T.a1[2 * kt + 1];
        h[kt][0] = pack_bf16(fmaxf(c0[0], 0.f), fmaxf(c0[1], 0.f));
        h[kt][1] = pack_bf16(fmaxf(c0[2], 0.f), fmaxf(c0[3], 0.f));
        h[kt][2] = pack_bf16(fmaxf(c1[0], 0.f), fmaxf(c1[1], 0.f));
        h[kt][3] = pack_bf16(fmaxf(c1[2], 0.f), fmaxf(c1[3], 0.f));
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const float bl = __ldg(M.b2 + nt * 8 + 2 * t), bh = __ldg(M.b2 + nt * 8 + 2 * t + 1);
        T.a2[nt][0] = bl; T.a2[nt][1] = bh; T.a2[nt][2] = bl; T.a2[nt][3] = bh;
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            unsigned b0, b1;
            load_bfrag(M.w2, 4, nt, kt, lane, b0, b1);
            mma_bf16(T.a2[nt], h[kt], b0, b1);
        }
    }
    // layer 3: FP32 dot of ReLU(a2) with w3, partial per lane, quad reduction
    float z0 = 0.f, z1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const float wl = __bfloat162float(M.w3[nt * 8 + 2 * t]), wh = __bfloat162float(M.w3[nt * 8 + 2 * t + 1]);
        z0 = fmaf(fmaxf(T.a2[nt][0], 0.f), wl, z0);
        z0 = fmaf(fmaxf(T.a2[nt][1], 0.f), wh, z0);
        z1 = fmaf(fmaxf(T.a2[nt][2], 0.f), wl, z1);
        z1 = fmaf(fmaxf(T.a2[nt][3], 0.f), wh, z1);
    }
    z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
    z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
    const float b3 = __ldg(M.b3);
    T.z[0] = z0 + b3;
    T.z[1] = z1 + b3;
}

// Inference-only forward of a 16-row tile: the same arithmetic as
// mlp_forward_tile, evaluated n-tile by n-tile so that only the layer-1
// activations (16 registers) stay live. z0, z1: logits of rows g and g + 8.
__device__ __forceinline__ void mlp_infer_tile(const MlpDev &M, const unsigned (&x)[4], int lane, float &z0,
                                               float &z1) {
    const int t = lane & 3;
    unsigned h[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const int nt = 2 * kt + half;
            const float bl = __ldg(M.b1 + nt * 8 + 2 * t), bh = __ldg(M.b1 + nt * 8 + 2 * t + 1);
            float c[4] = {bl, bh, bl, bh};
            unsigned b0, b1;
            load_bfrag(M.w1, 1, nt, 0, lane, b0, b1);
            mma_bf16(c, x, b0, b1);
            h[kt][2 * half] = pack_bf16(fmaxf(c[0], 0.f), fmaxf(c[1], 0.f));
            h[kt][2 * half + 1] = pack_bf16(fmaxf(c[2], 0.f), fmaxf(c[3], 0.f));
        }
    }
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const float bl = __ldg(M.b2 + nt * 8 + 2 * t), bh = __ldg(M.b2 + nt * 8 + 2 * t + 1);
        float c[4] = {bl, bh, bl, bh};
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            unsigned b0, b1;
            load_bfrag(M.w2, 4, nt, kt, lane, b0, b1);
            mma_bf16(c, h[kt], b0, b1);
        }
        const float wl = __bfloat162float(M.w3[nt * 8 + 2 * t]), wh = __bfloat162float(M.w3[nt * 8 + 2 * t + 1]);
        s0 = fmaf(fmaxf(c[0], 0.f), wl, s0);
        s0 = fmaf(fmaxf(c[1], 0.f), wh, s0);
        s1 = fmaf(fmaxf(c[2], 0.f), wl, s1);
        s1 = fmaf(fmaxf(c[3], 0.f), wh, s1);
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    const float b3 = __ldg(M.b3);
    z0 = s0 + b3;
    z1 = s1 + b3;
}

// A registers of a 16 x 16 BF16 tile stored row-major in shared memory.
__device__ __forceinline__ void load_a_smem(const __nv_bfloat16 *X, int lane, unsigned (&a)[4]) {
    const int g = lane >> 2, t = lane & 3;
    a[0] = *reinterpret_cast<const unsigned *>(X + g * 16 + 2 * t);
    a[1] = *reinterpret_cast<const unsigned *>(X + (g + 8) * 16 + 2 * t);
    a[2] = *reinterpret_cast<const unsigned *>(X + g * 16 + 2 * t + 8);
    a[3] = *reinterpret_cast<const unsigned *>(X + (g + 8) * 16 + 2 * t + 8);
}

}  // namespace gdp

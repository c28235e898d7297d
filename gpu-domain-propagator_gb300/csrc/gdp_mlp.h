// gdp_mlp.h -- host side of the row-marking MLP (gdp_mlp.cu).
#pragma once

#include <cuda_runtime.h>

#include "gdp_ext.h"
#include "gdp_mlp.cuh"

namespace gdp {

// Parameter vector layout (FP32 master copy): W1 [64][16], b1 [64], W2 [64][64],
// b2 [64], w3 [64], b3 [1].
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpH * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpH;
constexpr int kMlpParams = kOffB3 + 1;  // 5313

class Mlp {
public:
    ~Mlp();
    GDP_RETCODE init(unsigned long long seed, int device);
    GDP_RETCODE get(float *params) const;
    GDP_RETCODE set(const float *params);
    // x: n x 16 FP32 (host), rounded to BF16 on the device; z: n logits (host).
    GDP_RETCODE forward(int n, const float *x, float *z);
    // Gradient and loss of the weighted BCE at the current weights (host arrays).
    GDP_RETCODE gradient(int n, const float *x, const float *y, const float *w, float *grad, float *loss);
    // Adam over shuffled minibatches (host samples uploaded once).
    GDP_RETCODE train(int n, const float *x, const float *y, const float *w, int epochs, int batch, float lr,
                      unsigned long long seed, float *final_loss);
    MlpDev dev() const;

    int device = 0;
    cudaStream_t stream = nullptr;
    float *p = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *loss = nullptr;
    __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w2t = nullptr, *w3 = nullptr;
    int step = 0;

private:
    GDP_RETCODE refresh_bf16();
};

}  // namespace gdp

// The C-ABI handle (gdp_ext.h).
struct gdp_mlp {
    gdp::Mlp impl;
};

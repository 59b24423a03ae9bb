// The expansion-order selector's network: a small MLP in FP32.
//
// Input: kMlpIn pair features (normalised with stored means and inverse
// standard deviations); three hidden layers of kMlpH ReLU units; output: the
// predicted log10 of the M2L truncation error of the pair at expansion orders
// kQmin..kQmax (one output per order).
//
// Parameter blob layout (floats):
//   mean[In], istd[In], W1[H][In], b1[H], W2[H][H], b2[H], W3[H][H], b3[H],
//   W4[Q][H], b4[Q]
#pragma once

#include "internal.h"

namespace fmm {

constexpr int kMlpIn = 17;
constexpr int kMlpH = 64;
constexpr int kQmin = 2;
constexpr int kQmax = 12;
constexpr int kMlpOut = kQmax - kQmin + 1;

constexpr int kOffMean = 0;
constexpr int kOffIstd = kOffMean + kMlpIn;
constexpr int kOffW1 = kOffIstd + kMlpIn;
constexpr int kOffB1 = kOffW1 + kMlpH * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpH * kMlpH;
constexpr int kOffW4 = kOffB3 + kMlpH;
constexpr int kOffB4 = kOffW4 + kMlpOut * kMlpH;
constexpr int kMlpParams = kOffB4 + kMlpOut;

// Dense layer out[o] = b[o] + sum_k W[o][k] in[k]; the weights are read
// identically by all threads (broadcast from shared memory).
template <int NOUT, int NIN, bool RELU>
__device__ __forceinline__ void mlp_layer(const float* __restrict__ W, const float* __restrict__ b, const float* in,
                                          float* out) {
#pragma unroll 4
    for (int o = 0; o < NOUT; ++o) {
        float a = b[o];
#pragma unroll
        for (int k = 0; k < NIN; ++k) a = fmaf(W[o * NIN + k], in[k], a);
        out[o] = RELU ? fmaxf(a, 0.0f) : a;
    }
}

// Forward pass of one sample; P points at the parameter blob.
__device__ __forceinline__ void mlp_forward(const float* __restrict__ P, const float* x, float* y) {
    float in[kMlpIn], h1[kMlpH], h2[kMlpH];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) in[k] = (x[k] - P[kOffMean + k]) * P[kOffIstd + k];
    mlp_layer<kMlpH, kMlpIn, true>(P + kOffW1, P + kOffB1, in, h1);
    mlp_layer<kMlpH, kMlpH, true>(P + kOffW2, P + kOffB2, h1, h2);
    mlp_layer<kMlpH, kMlpH, true>(P + kOffW3, P + kOffB3, h2, h1);
    mlp_layer<kMlpOut, kMlpH, false>(P + kOffW4, P + kOffB4, h1, y);
}

// Features of the pair (target i, source j); P = order of the stored norms.
// Source norms of orders above kFeatOrders are not used (fixed at -40), so
// training (moments to order 12) and use (moments to the call's expansion
// order, at least kFeatOrders) see the same inputs.
constexpr int kFeatOrders = 10;
__device__ __forceinline__ void selector_features(const TreeDev& t, const float* __restrict__ lnorm,
                                                  const float* __restrict__ dmin, int P, int i, int j, float* x) {
    const double dx = t.cx[i] - t.cx[j], dy = t.cy[i] - t.cy[j], dz = t.cz[i] - t.cz[j];
    const double R = sqrt(dx * dx + dy * dy + dz * dz);
    const float lR = (float)log10(R);
    x[0] = (float)(1.7320508075688772 * (t.r[i] + t.r[j]) / R);
    x[1] = log2f((float)(t.r[j] / t.r[i]));
    x[2] = log2f((float)t.count[i]);
    for (int k = 0; k <= kQmax; ++k)
        x[3 + k] = (k <= P && k <= kFeatOrders) ? fmaxf(lnorm[(size_t)j * (P + 1) + k] - (float)(k + 2) * lR, -40.0f)
                                                : -40.0f;
    x[16] = fminf(dmin[i] * dmin[j] * (float)R, 30.0f) * (1.0f / 30.0f);
}

}  // namespace fmm

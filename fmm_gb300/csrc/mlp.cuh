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

// Inference layout of the parameters in shared memory (floats): the blob
// with W1's rows padded from kMlpIn to kMlpInP entries so that every weight
// row starts on a 16-byte boundary and is read as float4, and W4/b4 padded to
// kMlpOutP rows (zeros) so outputs come in blocks of four.
constexpr int kMlpInP = 20;
constexpr int kMlpOutP = 12;
constexpr int kSOffMean = 0;
constexpr int kSOffIstd = kSOffMean + kMlpIn;
constexpr int kSOffW1 = 36;
constexpr int kSOffB1 = kSOffW1 + kMlpH * kMlpInP;
constexpr int kSOffW2 = kSOffB1 + kMlpH;
constexpr int kSOffB2 = kSOffW2 + kMlpH * kMlpH;
constexpr int kSOffW3 = kSOffB2 + kMlpH;
constexpr int kSOffB3 = kSOffW3 + kMlpH * kMlpH;
constexpr int kSOffW4 = kSOffB3 + kMlpH;
constexpr int kSOffB4 = kSOffW4 + kMlpOutP * kMlpH;
constexpr int kMlpSmem = kSOffB4 + kMlpOutP;
static_assert(kSOffW2 % 4 == 0 && kSOffW3 % 4 == 0 && kSOffW4 % 4 == 0 && kMlpSmem % 4 == 0, "float4 rows");
static_assert(kSOffW4 - kSOffB1 == kOffW4 - kOffB1, "b1 .. b3 keep the blob's relative layout");

// Block-cooperative copy of the parameter blob into the inference layout.
__device__ __forceinline__ void mlp_stage(const float* __restrict__ P, float* S) {
    for (int e = threadIdx.x; e < kMlpSmem; e += blockDim.x) {
        float v = 0.0f;
        if (e < 2 * kMlpIn) {
            v = P[kOffMean + e];
        } else if (e >= kSOffW1 && e < kSOffB1) {
            const int o = (e - kSOffW1) / kMlpInP, k = (e - kSOffW1) % kMlpInP;
            v = k < kMlpIn ? P[kOffW1 + o * kMlpIn + k] : 0.0f;
        } else if (e >= kSOffB1 && e < kSOffW4) {
            v = P[kOffB1 + (e - kSOffB1)];
        } else if (e >= kSOffW4 && e < kSOffW4 + kMlpOut * kMlpH) {
            v = P[kOffW4 + (e - kSOffW4)];
        } else if (e >= kSOffB4 && e < kSOffB4 + kMlpOut) {
            v = P[kOffB4 + (e - kSOffB4)];
        }
        S[e] = v;
    }
}

// One dense layer out[o] = act(b[o] + W[o] . in), four outputs at a time
// (eight independent FMA chains), with `in` in registers (compile-time
// indices) and the outputs stored to this thread's column of the shared
// activation buffer (act[o * stride]), the only dynamically indexed array.
template <int NIN, bool RELU>
__device__ __forceinline__ void mlp_layer_smem(const float* W, const float* b, int nout, const float (&in)[NIN],
                                               float* act, int stride) {
#pragma unroll 1
    for (int o = 0; o < nout; o += 4) {
        const float4* w0 = reinterpret_cast<const float4*>(W + o * NIN);
        float a[4][2];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            a[r][0] = b[o + r];
            a[r][1] = 0.0f;
        }
#pragma unroll
        for (int k = 0; k < NIN / 4; ++k) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float4 w = w0[r * (NIN / 4) + k];
                a[r][0] = fmaf(w.x, in[4 * k], a[r][0]);
                a[r][1] = fmaf(w.y, in[4 * k + 1], a[r][1]);
                a[r][0] = fmaf(w.z, in[4 * k + 2], a[r][0]);
                a[r][1] = fmaf(w.w, in[4 * k + 3], a[r][1]);
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const float v = a[r][0] + a[r][1];
            act[(o + r) * stride] = RELU ? fmaxf(v, 0.0f) : v;
        }
    }
}

template <int N>
__device__ __forceinline__ void mlp_load_act(const float* act, int stride, float (&v)[N]) {
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = act[k * stride];
}

// Forward pass with the weights in the inference layout S and a per-thread
// activation column act (kMlpH entries at stride `stride`); the kMlpOut
// outputs are left in act[0 .. kMlpOut-1] (same stride).
__device__ __forceinline__ void mlp_forward_smem(const float* S, float* act, int stride, const float* x) {
    float in[kMlpInP];
#pragma unroll
    for (int k = 0; k < kMlpInP; ++k) in[k] = k < kMlpIn ? (x[k] - S[kSOffMean + k]) * S[kSOffIstd + k] : 0.0f;
    mlp_layer_smem<kMlpInP, true>(S + kSOffW1, S + kSOffB1, kMlpH, in, act, stride);
    float h[kMlpH];
    mlp_load_act(act, stride, h);
    mlp_layer_smem<kMlpH, true>(S + kSOffW2, S + kSOffB2, kMlpH, h, act, stride);
    mlp_load_act(act, stride, h);
    mlp_layer_smem<kMlpH, true>(S + kSOffW3, S + kSOffB3, kMlpH, h, act, stride);
    mlp_load_act(act, stride, h);
    mlp_layer_smem<kMlpH, false>(S + kSOffW4, S + kSOffB4, kMlpOutP, h, act, stride);
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

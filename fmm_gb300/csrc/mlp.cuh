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

// Inference layout of the parameters (floats): the blob
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

// The device copy of the parameters holds the blob followed (at kMlpInfOff)
// by the inference layout above, written once by k_mlp_stage_global.
constexpr int kMlpInfOff = (kMlpParams + 3) / 4 * 4;
constexpr int kMlpBufFloats = kMlpInfOff + kMlpSmem;

namespace {
__global__ void k_mlp_stage_global(float* buf) { mlp_stage(buf, buf + kMlpInfOff); }
}  // namespace

// Warp-cooperative inference on up to 32 samples (weights stationary in
// registers): lane l owns hidden units 2l and 2l+1 of every layer and streams
// the samples' input rows from shared memory (broadcast reads), so every
// weight is read once per batch instead of once per sample.  Per-warp
// scratch: X[32][kMlpInP] (normalised inputs, filled by the caller), two
// activation buffers [32][kMlpH] and Y[32][kMlpOutP] (outputs).
constexpr int kWarpMlpFloats = 32 * (kMlpInP + 2 * kMlpH + kMlpOutP);

template <int NIN>
__device__ __forceinline__ void warp_mlp_layer(const float* __restrict__ W, const float* __restrict__ b, const float* in,
                                               float* outp, int cnt, int u0, bool relu) {
    float wa[NIN], wb[NIN];
    const float4* ra = reinterpret_cast<const float4*>(W + u0 * NIN);
    const float4* rb = reinterpret_cast<const float4*>(W + (u0 + 1) * NIN);
#pragma unroll
    for (int k = 0; k < NIN / 4; ++k) {
        const float4 x = __ldg(ra + k), y = __ldg(rb + k);
        wa[4 * k] = x.x; wa[4 * k + 1] = x.y; wa[4 * k + 2] = x.z; wa[4 * k + 3] = x.w;
        wb[4 * k] = y.x; wb[4 * k + 1] = y.y; wb[4 * k + 2] = y.z; wb[4 * k + 3] = y.w;
    }
    const float ba = __ldg(b + u0), bb = __ldg(b + u0 + 1);
    // two samples per step: eight independent FMA chains
    for (int s = 0; s < cnt; s += 2) {
        const bool two = s + 1 < cnt;
        const float4* x4 = reinterpret_cast<const float4*>(in + s * NIN);
        const float4* y4 = reinterpret_cast<const float4*>(in + (two ? s + 1 : s) * NIN);
        float a0 = ba, c0 = 0.0f, a1 = bb, c1 = 0.0f;
        float d0 = ba, e0 = 0.0f, d1 = bb, e1 = 0.0f;
#pragma unroll
        for (int k = 0; k < NIN / 4; ++k) {
            const float4 x = x4[k], y = y4[k];
            a0 = fmaf(wa[4 * k], x.x, a0);
            c0 = fmaf(wa[4 * k + 1], x.y, c0);
            a1 = fmaf(wb[4 * k], x.x, a1);
            c1 = fmaf(wb[4 * k + 1], x.y, c1);
            d0 = fmaf(wa[4 * k], y.x, d0);
            e0 = fmaf(wa[4 * k + 1], y.y, e0);
            d1 = fmaf(wb[4 * k], y.x, d1);
            e1 = fmaf(wb[4 * k + 1], y.y, e1);
            a0 = fmaf(wa[4 * k + 2], x.z, a0);
            c0 = fmaf(wa[4 * k + 3], x.w, c0);
            a1 = fmaf(wb[4 * k + 2], x.z, a1);
            c1 = fmaf(wb[4 * k + 3], x.w, c1);
            d0 = fmaf(wa[4 * k + 2], y.z, d0);
            e0 = fmaf(wa[4 * k + 3], y.w, e0);
            d1 = fmaf(wb[4 * k + 2], y.z, d1);
            e1 = fmaf(wb[4 * k + 3], y.w, e1);
        }
        float v0 = a0 + c0, v1 = a1 + c1, w0 = d0 + e0, w1 = d1 + e1;
        if (relu) {
            v0 = fmaxf(v0, 0.0f);
            v1 = fmaxf(v1, 0.0f);
            w0 = fmaxf(w0, 0.0f);
            w1 = fmaxf(w1, 0.0f);
        }
        *reinterpret_cast<float2*>(outp + s * kMlpH + u0) = make_float2(v0, v1);
        if (two) *reinterpret_cast<float2*>(outp + (s + 1) * kMlpH + u0) = make_float2(w0, w1);
    }
}

__device__ __forceinline__ void warp_mlp(const float* __restrict__ S, float* X, float* Ha, float* Hb, float* Y,
                                         int cnt, int lane) {
    const int u0 = 2 * lane;
    warp_mlp_layer<kMlpInP>(S + kSOffW1, S + kSOffB1, X, Ha, cnt, u0, true);
    __syncwarp();
    warp_mlp_layer<kMlpH>(S + kSOffW2, S + kSOffB2, Ha, Hb, cnt, u0, true);
    __syncwarp();
    warp_mlp_layer<kMlpH>(S + kSOffW3, S + kSOffB3, Hb, Ha, cnt, u0, true);
    __syncwarp();
    if (lane < kMlpOut) {
        float w[kMlpH];
        const float4* r = reinterpret_cast<const float4*>(S + kSOffW4 + lane * kMlpH);
#pragma unroll
        for (int k = 0; k < kMlpH / 4; ++k) {
            const float4 x = __ldg(r + k);
            w[4 * k] = x.x; w[4 * k + 1] = x.y; w[4 * k + 2] = x.z; w[4 * k + 3] = x.w;
        }
        const float b = __ldg(S + kSOffB4 + lane);
        for (int s = 0; s < cnt; ++s) {
            const float4* x4 = reinterpret_cast<const float4*>(Ha + s * kMlpH);
            float a = b, c = 0.0f;
#pragma unroll
            for (int k = 0; k < kMlpH / 4; ++k) {
                const float4 x = x4[k];
                a = fmaf(w[4 * k], x.x, a);
                c = fmaf(w[4 * k + 1], x.y, c);
                a = fmaf(w[4 * k + 2], x.z, a);
                c = fmaf(w[4 * k + 3], x.w, c);
            }
            Y[s * kMlpOutP + lane] = a + c;
        }
    }
    __syncwarp();
}

// Normalised, padded network input of one sample (kMlpInP floats).
__device__ __forceinline__ void mlp_input(const float* __restrict__ S, const float* x, float* row) {
#pragma unroll
    for (int k = 0; k < kMlpInP; ++k) row[k] = k < kMlpIn ? (x[k] - __ldg(S + kSOffMean + k)) * __ldg(S + kSOffIstd + k) : 0.0f;
}

// Features of the pair (target i, source j); P = order of the stored norms.
// Source norms of orders above kFeatOrders are not used (fixed at -40), so
// training (moments to order 12) and use (moments to the call's expansion
// order, at least kFeatOrders) see the same inputs.
constexpr int kFeatOrders = 10;
__device__ __forceinline__ void selector_features(const TreeDev& t, const float* __restrict__ lnorm,
                                                  const float* __restrict__ dmin, int P, int i, int j, float* x) {
    // FP32 is ample for network inputs (the FP64 pipe is the scarce one)
    const float dx = (float)(t.cx[i] - t.cx[j]), dy = (float)(t.cy[i] - t.cy[j]), dz = (float)(t.cz[i] - t.cz[j]);
    const float R = sqrtf(dx * dx + dy * dy + dz * dz);
    const float lR = log10f(R);
    const float ri = (float)t.r[i], rj = (float)t.r[j];
    x[0] = 1.7320508f * (ri + rj) / R;
    x[1] = log2f(rj / ri);
    x[2] = log2f((float)t.count[i]);
    for (int k = 0; k <= kQmax; ++k)
        x[3 + k] = (k <= P && k <= kFeatOrders) ? fmaxf(lnorm[(size_t)j * (P + 1) + k] - (float)(k + 2) * lR, -40.0f)
                                                : -40.0f;
    x[16] = fminf(dmin[i] * dmin[j] * R, 30.0f) * (1.0f / 30.0f);
}

}  // namespace fmm

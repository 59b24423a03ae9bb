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

#include <cuda_fp16.h>

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

// Tensor-core inference (warp-level m16n8k16 MMA, FP16 operands, FP32
// accumulation): per layer, the weights as B fragments in lane order (uint2
// per lane and (k-tile, n-tile)), inputs padded to 32, outputs of the last
// layer padded to 16; biases in FP32.
constexpr int kTcK1 = 2, kTcKH = kMlpH / 16, kTcN = kMlpH / 8, kTcN4 = 2;  // k-tiles / n-tiles
constexpr int kTcF1 = 0, kTcF2 = kTcF1 + kTcK1 * kTcN, kTcF3 = kTcF2 + kTcKH * kTcN, kTcF4 = kTcF3 + kTcKH * kTcN;
constexpr int kTcFrags = kTcF4 + kTcKH * kTcN4;
constexpr int kTcBias = 3 * kMlpH + 16;

// The device copy of the parameters holds the blob followed (at kMlpInfOff)
// by the FP32 inference layout above, the FP32 biases and the FP16 weight
// fragments; all written once by k_mlp_stage_global.
constexpr int kMlpInfOff = (kMlpParams + 3) / 4 * 4;
constexpr int kTcBiasOff = kMlpInfOff + kMlpSmem;
constexpr int kTcFragOff = kTcBiasOff + kTcBias;  // uint2 entries from here
constexpr int kMlpBufFloats = kTcFragOff + 2 * 32 * kTcFrags;
static_assert(kTcFragOff % 2 == 0, "8-byte fragments");

__device__ __forceinline__ uint32_t pack_half2(float lo, float hi) {
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

namespace {
__global__ void k_mlp_stage_global(float* buf) {
    mlp_stage(buf, buf + kMlpInfOff);
    const float* P = buf;
    float* bias = buf + kTcBiasOff;
    for (int e = threadIdx.x; e < kTcBias; e += blockDim.x) {
        float v = 0.0f;
        if (e < kMlpH) v = P[kOffB1 + e];
        else if (e < 2 * kMlpH) v = P[kOffB2 + e - kMlpH];
        else if (e < 3 * kMlpH) v = P[kOffB3 + e - 2 * kMlpH];
        else if (e - 3 * kMlpH < kMlpOut) v = P[kOffB4 + e - 3 * kMlpH];
        bias[e] = v;
    }
    uint2* frag = reinterpret_cast<uint2*>(buf + kTcFragOff);
    for (int e = threadIdx.x; e < 32 * kTcFrags; e += blockDim.x) {
        const int fi = e >> 5, lane = e & 31, g = lane >> 2, t = lane & 3;
        int layer, kt, nt;
        if (fi < kTcF2) { layer = 1; kt = (fi - kTcF1) / kTcN; nt = (fi - kTcF1) % kTcN; }
        else if (fi < kTcF3) { layer = 2; kt = (fi - kTcF2) / kTcN; nt = (fi - kTcF2) % kTcN; }
        else if (fi < kTcF4) { layer = 3; kt = (fi - kTcF3) / kTcN; nt = (fi - kTcF3) % kTcN; }
        else { layer = 4; kt = (fi - kTcF4) / kTcN4; nt = (fi - kTcF4) % kTcN4; }
        const int nn = 8 * nt + g, k0 = 16 * kt + 2 * t;
        auto w = [&](int k) -> float {
            if (layer == 1) return (k < kMlpIn) ? P[kOffW1 + nn * kMlpIn + k] : 0.0f;
            if (layer == 2) return P[kOffW2 + nn * kMlpH + k];
            if (layer == 3) return P[kOffW3 + nn * kMlpH + k];
            return nn < kMlpOut ? P[kOffW4 + nn * kMlpH + k] : 0.0f;
        };
        frag[e] = make_uint2(pack_half2(w(k0), w(k0 + 1)), pack_half2(w(k0 + 8), w(k0 + 9)));
    }
}
}  // namespace

__device__ __forceinline__ void mma_16816(float (&c)[4], const uint32_t (&a)[4], uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// One hidden layer on a 16-sample tile: A fragments in (KT k-tiles), ReLU'd
// outputs packed as the next layer's A fragments (kTcKH k-tiles); the
// m16n8 accumulator layout of n-tiles 2k and 2k+1 is exactly the m16k16 A
// layout of k-tile k.
template <int KT>
__device__ __forceinline__ void tc_hidden(const uint2* __restrict__ frag, const float* __restrict__ bias,
                                          const uint32_t (&a)[KT][4], uint32_t (&o)[kTcKH][4], int lane) {
    const int t = lane & 3;
    float c[kTcN][4];
#pragma unroll
    for (int nt = 0; nt < kTcN; ++nt) {
        const float b0 = __ldg(bias + 8 * nt + 2 * t), b1 = __ldg(bias + 8 * nt + 2 * t + 1);
        c[nt][0] = b0;
        c[nt][1] = b1;
        c[nt][2] = b0;
        c[nt][3] = b1;
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
#pragma unroll
        for (int nt = 0; nt < kTcN; ++nt) mma_16816(c[nt], a[kt], __ldg(frag + (kt * kTcN + nt) * 32 + lane));
#pragma unroll
    for (int k = 0; k < kTcKH; ++k) {
        o[k][0] = pack_half2(fmaxf(c[2 * k][0], 0.0f), fmaxf(c[2 * k][1], 0.0f));
        o[k][1] = pack_half2(fmaxf(c[2 * k][2], 0.0f), fmaxf(c[2 * k][3], 0.0f));
        o[k][2] = pack_half2(fmaxf(c[2 * k + 1][0], 0.0f), fmaxf(c[2 * k + 1][1], 0.0f));
        o[k][3] = pack_half2(fmaxf(c[2 * k + 1][2], 0.0f), fmaxf(c[2 * k + 1][3], 0.0f));
    }
}

constexpr int kWarpTcFloats = 32 * (kMlpInP + kMlpOutP);  // per-warp scratch: X then Y

// Warp-level tensor-core inference on up to 32 samples: X[32][kMlpInP]
// normalised inputs (rows >= cnt ignored), outputs to Y[32][kMlpOutP]
// (first kMlpOut columns).  buf is the device parameter buffer.
__device__ __forceinline__ void warp_mlp_tc(const float* __restrict__ buf, const float* X, float* Y, int cnt,
                                            int lane) {
    const int g = lane >> 2, t = lane & 3;
    const uint2* frag = reinterpret_cast<const uint2*>(buf + kTcFragOff);
    const float* bias = buf + kTcBiasOff;
    for (int m0 = 0; m0 < cnt; m0 += 16) {
        const float* x0 = X + (m0 + g) * kMlpInP;
        const float* x1 = X + (m0 + g + 8) * kMlpInP;
        uint32_t a1[kTcK1][4];
#pragma unroll
        for (int kt = 0; kt < kTcK1; ++kt) {
            const int k = 16 * kt + 2 * t;
            auto ld = [&](const float* x, int kk) { return kk < kMlpInP ? x[kk] : 0.0f; };
            a1[kt][0] = pack_half2(ld(x0, k), ld(x0, k + 1));
            a1[kt][1] = pack_half2(ld(x1, k), ld(x1, k + 1));
            a1[kt][2] = pack_half2(ld(x0, k + 8), ld(x0, k + 9));
            a1[kt][3] = pack_half2(ld(x1, k + 8), ld(x1, k + 9));
        }
        uint32_t h1[kTcKH][4], h2[kTcKH][4];
        tc_hidden<kTcK1>(frag + kTcF1 * 32, bias, a1, h1, lane);
        tc_hidden<kTcKH>(frag + kTcF2 * 32, bias + kMlpH, h1, h2, lane);
        tc_hidden<kTcKH>(frag + kTcF3 * 32, bias + 2 * kMlpH, h2, h1, lane);
        float c[kTcN4][4];
#pragma unroll
        for (int nt = 0; nt < kTcN4; ++nt) {
            const float b0 = __ldg(bias + 3 * kMlpH + 8 * nt + 2 * t), b1 = __ldg(bias + 3 * kMlpH + 8 * nt + 2 * t + 1);
            c[nt][0] = b0;
            c[nt][1] = b1;
            c[nt][2] = b0;
            c[nt][3] = b1;
        }
#pragma unroll
        for (int kt = 0; kt < kTcKH; ++kt)
#pragma unroll
            for (int nt = 0; nt < kTcN4; ++nt) mma_16816(c[nt], h1[kt], __ldg(frag + (kTcF4 + kt * kTcN4 + nt) * 32 + lane));
#pragma unroll
        for (int nt = 0; nt < kTcN4; ++nt) {
            const int col = 8 * nt + 2 * t;
            if (col < kMlpOutP) {
                Y[(m0 + g) * kMlpOutP + col] = c[nt][0];
                Y[(m0 + g + 8) * kMlpOutP + col] = c[nt][2];
            }
            if (col + 1 < kMlpOutP) {
                Y[(m0 + g) * kMlpOutP + col + 1] = c[nt][1];
                Y[(m0 + g + 8) * kMlpOutP + col + 1] = c[nt][3];
            }
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

// The same features from the FP32 node data of the learned list build
// (centres as double-float pairs, rmax in chi.w, half-width in clo.w).
__device__ __forceinline__ void selector_features_f32(const float4* __restrict__ chi, const float4* __restrict__ clo,
                                                      const int32_t* __restrict__ count,
                                                      const float* __restrict__ lnorm,
                                                      const float* __restrict__ dmin, int P, int i, int j, float* x) {
    const float4 ci = chi[i], cj = chi[j], li = clo[i], lj = clo[j];
    const float dx = (ci.x - cj.x) + (li.x - lj.x), dy = (ci.y - cj.y) + (li.y - lj.y),
                dz = (ci.z - cj.z) + (li.z - lj.z);
    const float R = sqrtf(dx * dx + dy * dy + dz * dz);
    const float lR = log10f(R);
    const float ri = li.w, rj = lj.w;
    x[0] = 1.7320508f * (ri + rj) / R;
    x[1] = log2f(rj / ri);
    x[2] = log2f((float)count[i]);
    for (int k = 0; k <= kQmax; ++k)
        x[3 + k] = (k <= P && k <= kFeatOrders) ? fmaxf(lnorm[(size_t)j * (P + 1) + k] - (float)(k + 2) * lR, -40.0f)
                                                : -40.0f;
    x[16] = fminf(dmin[i] * dmin[j] * R, 30.0f) * (1.0f / 30.0f);
}

}  // namespace fmm

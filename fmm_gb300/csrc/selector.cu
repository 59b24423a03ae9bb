// Learned expansion-order selector: features, training data, training and
// batched inference kernels.
//
// For a far pair (target cell i, source cell j) the network predicts
// log10 E_q, the RMS error of the field (order-1 components) that the pair's
// M2L + L2P contribution carries when truncated at expansion order q, for
// q = 2..12.  Training labels are measured by the method itself: the same
// reduced-basis translation at every order is evaluated at sample particles of
// the target cell and compared with the FP64 direct sum over the source cell's
// particles.  During list generation the selector accepts a pair at the
// lowest order whose predicted error fits the pair's error budget, or refines
// it (see tree.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "dispatch.cuh"
#include "internal.h"
#include "mlp.cuh"
#include "pair.cuh"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

__host__ __device__ constexpr int rbase_s(int n) { return n == 0 ? 0 : 1 + 3 * (n - 1) * n / 2; }
__host__ __device__ constexpr int ridx_s(int t, int u, int v) {
    return rbase_s(t + u + v) + (v == 0 ? 0 : (v == 1 ? t + u + v + 1 : 2 * (t + u + v) + 1)) + u;
}
__device__ __forceinline__ int qcomp_s(int q) {
    int k = 0;
    while ((k + 1) * (k + 1) <= q) ++k;
    const int l = q - k * k;
    const int z = l <= k ? 0 : 1;
    const int y = z == 0 ? l : l - (k + 1);
    return (k - y - z) | (y << 8) | (z << 16) | (k << 24);
}

// Per node: log10 of the norm of the reduced source weights of each order,
// and the smallest damping factor of the node's particles.
__global__ void k_node_norms(int M, int P, const double* __restrict__ wred, const TreeDev t,
                             const double* __restrict__ sd, float* __restrict__ lnorm, float* __restrict__ dmin) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= M) return;
    const int nr = (P + 1) * (P + 1);
    for (int k = 0; k <= P; ++k) {
        double s = 0.0;
        for (int q = k * k; q < (k + 1) * (k + 1); ++q) {
            const double v = wred[(size_t)node * nr + q];
            s += v * v;
        }
        lnorm[(size_t)node * (P + 1) + k] = (float)log10(sqrt(s) + 1e-300);
    }
    // leaves: smallest damping factor of their particles; internal nodes
    // start at +inf and take the minimum of their leaves (k_dmin_up)
    float dm = sd ? __int_as_float(0x7f800000) : 0.0f;
    if (sd && t.is_leaf[node]) {
        double v = 1e300;
        const int s0 = t.start[node], c = t.count[node];
        for (int q = s0; q < s0 + c; ++q) v = fmin(v, sd[q]);
        dm = (float)v;
    }
    dmin[node] = dm;
}

// Propagates leaf minima to all ancestors.  Damping factors are positive, so
// the order of their float bit patterns as signed integers is their order.
__global__ void k_dmin_up(int M, const TreeDev t, float* __restrict__ dmin) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= M || !t.is_leaf[node]) return;
    const int v = __float_as_int(dmin[node]);
    for (int a = t.parent[node]; a >= 0; a = t.parent[a]) atomicMin(reinterpret_cast<int*>(dmin + a), v);
}

// Order-preserving map of floats to ints (for atomicMin on any sign).
__device__ __forceinline__ int ordered_int(float f) {
    const int b = __float_as_int(f);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float ordered_float(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// Per node: the smallest of its leaves' scales (each leaf's mean log10 local
// field over its sample particles), by atomicMin into every ancestor.
__global__ void k_scale_up(int M, const TreeDev t, const float* __restrict__ lmean, int* __restrict__ mn) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= M || !t.is_leaf[node]) return;
    const int m = ordered_int(lmean[node]);
    for (int a = node; a >= 0; a = t.parent[a]) atomicMin(mn + a, m);
}

// log10 error budget of a far pair with the node as target: base + the
// node's scale.  A node's particles differ in field strength; the weakest
// leaf of a node (the tail of a cluster, a particle far from its
// neighbours) sets how much absolute error that node's far pairs may carry.
__global__ void k_node_budget(int M, float base, const int* __restrict__ mn, float* __restrict__ budget) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= M) return;
    budget[node] = base + ordered_float(mn[node]);
}

}  // namespace

// Per-node log10 error budgets of the learned selector (see k_node_budget):
// leaf field scales from the FP32 records, minimum over each subtree.
int selector_node_budgets(Workspace& ws, const Particles& P, const TreeDev& t, float base, cudaStream_t st) {
    const int M = t.num_nodes;
    FMM_TRY(ws.sel_budget.ensure(sizeof(float) * 4 * (size_t)M));
    float* lscale = ws.sel_budget.as<float>() + M;  // leaf means, then leaf minima
    int* mn = reinterpret_cast<int*>(lscale + 2 * (size_t)M);
    FMM_CUDA_TRY(cudaMemsetAsync(mn, 0x7f, sizeof(int) * (size_t)M, st));
    FMM_TRY(launch_leaf_field_scale(ws, P, t, lscale, st));
    count_launches(1);
    k_scale_up<<<grid_for(M, 128), 128, 0, st>>>(M, t, lscale, mn);
    count_launches(1);
    k_node_budget<<<grid_for(M, 256), 256, 0, st>>>(M, base, mn, ws.sel_budget.as<float>());
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

namespace {

// ---------------------------------------------------------------- labels
constexpr int kLabT = 8;  // sample particles per target cell

// One warp per sampled pair (FP64).  Shared per warp: restricted tensor (two
// buffers), reduced weights, reduced and full local expansions, exact fields,
// scaled powers of the sample particles' offsets.
template <int M>
__global__ void k_pair_errors(const TreeDev t, int P, const int2* __restrict__ pairs, int npairs,
                              const double* __restrict__ sx, const double* __restrict__ sy,
                              const double* __restrict__ sz, const double* __restrict__ smc, int64_t n,
                              const double* __restrict__ wred, float* __restrict__ labels) {
    extern __shared__ double sm[];
    constexpr int NM = nT(M);
    const int N = 2 * P, nTr = rbase_s(N + 1), nr = (P + 1) * (P + 1), nq = nT(P);
    const int per_warp = 2 * nTr + nr + nr + nq + kLabT * 3 + kLabT * 3 * 13 + (N + 1);
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* TA = sm + wib * per_warp;
    double* TB = TA + nTr;
    double* ws = TB + nTr;
    double* Lr = ws + nr;
    double* Lf = Lr + nr;
    double* Fx = Lf + nq;
    double* ep = Fx + kLabT * 3;
    double* gsh = ep + kLabT * 3 * 13;
    const int pr = blockIdx.x * (blockDim.x >> 5) + wib;
    if (pr >= npairs) return;
    const int i = pairs[pr].x, j = pairs[pr].y;
    const int si = t.start[i], ci = t.count[i];
    const int sj = t.start[j], cj = t.count[j];
    const int nt = min(kLabT, ci);
    const double cxi = t.cx[i], cyi = t.cy[i], czi = t.cz[i];
    // sample targets, their offsets from the target centre as d^a / a!
    const int tt = lane >> 2, grp = lane & 3;
    for (int e = lane; e < nt * 3; e += 32) {
        const int ti = e / 3, c = e % 3;
        const int k = si + (int)((int64_t)ti * ci / nt);
        const double d = c == 0 ? sx[k] - cxi : (c == 1 ? sy[k] - cyi : sz[k] - czi);
        double* e3 = ep + (ti * 3 + c) * 13;
        e3[0] = 1.0;
        for (int a = 1; a <= P; ++a) e3[a] = e3[a - 1] * d / (double)a;
    }
    // exact field of the source cell's particles (undamped, FP64)
    {
        double acc[4] = {0, 0, 0, 0};
        if (tt < nt) {
            const int k = si + (int)((int64_t)tt * ci / nt);
            const double xt = sx[k], yt = sy[k], zt = sz[k];
            for (int q = sj + grp; q < sj + cj; q += 4) {
                double mc[NM];
#pragma unroll
                for (int s = 0; s < NM; ++s) mc[s] = smc[(size_t)s * n + q];
                pair_field<M, 1, double>(xt - sx[q], yt - sy[q], zt - sz[q], 0.0, DAMP_NONE, mc, acc);
            }
        }
#pragma unroll
        for (int c = 1; c < 4; ++c) {
            acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 1);
            acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 2);
        }
        if (grp == 0 && tt < nt)
            for (int c = 0; c < 3; ++c) Fx[tt * 3 + c] = acc[c + 1];
    }
    // restricted tensor of orders <= 2P at R = c_i - c_j (FP64, unscaled)
    const double X = cxi - t.cx[j], Y = cyi - t.cy[j], Z = czi - t.cz[j];
    const double rinv = 1.0 / sqrt(X * X + Y * Y + Z * Z), rinv2 = rinv * rinv;
    if (lane <= N) {
        double v = rinv, c = 1.0;
        for (int jj = 1; jj <= lane; ++jj) {
            v *= rinv2;
            c *= -(double)(2 * jj - 1);
        }
        gsh[lane] = c * v;
    }
    for (int s = lane; s < nr; s += 32) {
        ws[s] = wred[(size_t)j * nr + s];
        Lr[s] = 0.0;
    }
    __syncwarp();
    double* A = TA;
    double* B = TB;
    if (lane == 0) A[0] = gsh[N];
    __syncwarp();
    for (int lev = N - 1; lev >= 0; --lev) {
        const int lim = rbase_s(N - lev + 1);
        for (int e = lane; e < lim; e += 32) {
            double v;
            if (e == 0) {
                v = gsh[lev];
            } else {
                int n2 = 0;
                while (rbase_s(n2 + 1) <= e) ++n2;
                const int l = e - rbase_s(n2);
                const int vv = l <= n2 ? 0 : (l <= 2 * n2 ? 1 : 2);
                const int u = l - (vv == 0 ? 0 : (vv == 1 ? n2 + 1 : 2 * n2 + 1));
                const int tx = n2 - vv - u;
                if (tx > 0) {
                    v = X * A[ridx_s(tx - 1, u, vv)];
                    if (tx > 1) v += (double)(tx - 1) * A[ridx_s(tx - 2, u, vv)];
                } else if (u > 0) {
                    v = Y * A[ridx_s(0, u - 1, vv)];
                    if (u > 1) v += (double)(u - 1) * A[ridx_s(0, u - 2, vv)];
                } else {
                    v = Z * A[ridx_s(0, 0, vv - 1)];
                    if (vv > 1) v += (double)(vv - 1) * A[ridx_s(0, 0, vv - 2)];
                }
            }
            B[e] = v;
        }
        __syncwarp();
        double* tmp = A;
        A = B;
        B = tmp;
    }
    // source orders one at a time; after order q the truncated local
    // expansion is evaluated at the sample particles
    for (int k = 0; k <= P; ++k) {
        for (int f = lane; f < nr; f += 32) {
            const int cf = qcomp_s(f);
            const int fx = cf & 0xff, fy = (cf >> 8) & 0xff, fz = (cf >> 16) & 0xff;
            double a = 0.0;
            for (int s = k * k; s < (k + 1) * (k + 1); ++s) {
                const int cs = qcomp_s(s);
                a += ws[s] * A[ridx_s((cs & 0xff) + fx, ((cs >> 8) & 0xff) + fy, ((cs >> 16) & 0xff) + fz)];
            }
            Lr[f] += a;
        }
        __syncwarp();
        if (k < kQmin) continue;
        const int q = k;
        // full local expansion of orders <= q: reduced entries, then completion
        for (int e = lane; e < nT(q); e += 32) Lf[e] = 0.0;
        __syncwarp();
        for (int f = lane; f < (q + 1) * (q + 1); f += 32) {
            const int cf = qcomp_s(f);
            Lf[pidx(cf & 0xff, (cf >> 8) & 0xff, (cf >> 16) & 0xff)] = Lr[f];
        }
        __syncwarp();
        for (int fz = 2; fz <= q; ++fz) {
            for (int e = lane; e < (q - fz + 1) * (q - fz + 2) / 2; e += 32) {
                int w2 = 0;
                while ((w2 + 1) * (w2 + 2) / 2 <= e) ++w2;
                const int fy = e - w2 * (w2 + 1) / 2, fx = w2 - fy;
                Lf[pidx(fx, fy, fz)] = -Lf[pidx(fx + 2, fy, fz - 2)] - Lf[pidx(fx, fy + 2, fz - 2)];
            }
            __syncwarp();
        }
        // field at the sample particles: F_u = sum_w L_{u+w} d^w / w!
        double err2 = 0.0;
        {
            double F[3] = {0, 0, 0};
            if (tt < nt) {
                const double* ex = ep + (tt * 3 + 0) * 13;
                const double* ey = ep + (tt * 3 + 1) * 13;
                const double* ez = ep + (tt * 3 + 2) * 13;
                for (int w = grp; w < nT(q - 1); w += 4) {
                    int wo = 0;
                    while (nT(wo) <= w) ++wo;
                    const int l = w - nT(wo - 1);
                    int w2 = 0;
                    while ((w2 + 1) * (w2 + 2) / 2 <= l) ++w2;
                    const int wz = l - w2 * (w2 + 1) / 2, wy = w2 - wz, wx = wo - w2;
                    const double dp = ex[wx] * ey[wy] * ez[wz];
                    F[0] += Lf[pidx(wx + 1, wy, wz)] * dp;
                    F[1] += Lf[pidx(wx, wy + 1, wz)] * dp;
                    F[2] += Lf[pidx(wx, wy, wz + 1)] * dp;
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                F[c] += __shfl_xor_sync(0xffffffffu, F[c], 1);
                F[c] += __shfl_xor_sync(0xffffffffu, F[c], 2);
            }
            if (grp == 0 && tt < nt)
                for (int c = 0; c < 3; ++c) {
                    const double d = F[c] - Fx[tt * 3 + c];
                    err2 += d * d;
                }
        }
        for (int off = 4; off < 32; off <<= 1) err2 += __shfl_xor_sync(0xffffffffu, err2, off);
        // errors below 1e-14 (field units) are rounding noise of the FP64 sums
        if (lane == 0) labels[(size_t)pr * kMlpOut + (q - kQmin)] = (float)log10(fmax(sqrt(err2 / nt), 1e-14));
        __syncwarp();
    }
}

__global__ void k_pair_feats(const TreeDev t, const float* __restrict__ lnorm, const float* __restrict__ dmin, int P,
                             const int2* __restrict__ pairs, int npairs, float* __restrict__ feats) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npairs) return;
    float x[kMlpIn];
    selector_features(t, lnorm, dmin, P, pairs[q].x, pairs[q].y, x);
    for (int k = 0; k < kMlpIn; ++k) feats[(size_t)q * kMlpIn + k] = x[k];
}

__global__ void k_unpack_far(int64_t nfar, const uint64_t* __restrict__ sorted, int2* __restrict__ out) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= nfar) return;
    const uint64_t v = sorted[k];
    out[k] = make_int2((int)(v >> 36), (int)(v & 0xffffffffull));
}

// ---------------------------------------------------------------- training
constexpr int kTB = 64;  // samples per training block

// Forward and backward pass of kTB samples; gradients of the mean squared
// error (over samples of the whole batch and outputs) added to `grad`.
__global__ void __launch_bounds__(kTB) k_mlp_fwd_bwd(const float* __restrict__ params, const float* __restrict__ X,
                                                     const float* __restrict__ Y, const int* __restrict__ idx,
                                                     int nb, float inv_count, float* __restrict__ grad,
                                                     float* __restrict__ loss) {
    extern __shared__ float smf[];
    float* P = smf;                                   // parameters
    float* a0 = P + kMlpParams;                       // [kTB][In]   normalised inputs
    float* a1 = a0 + kTB * kMlpIn;                    // [kTB][H]
    float* a2 = a1 + kTB * kMlpH;
    float* a3 = a2 + kTB * kMlpH;
    float* d4 = a3 + kTB * kMlpH;                     // [kTB][Out]
    float* d3 = d4 + kTB * kMlpOut;                   // [kTB][H]
    float* d2 = d3 + kTB * kMlpH;
    float* d1 = d2 + kTB * kMlpH;
    for (int e = threadIdx.x; e < kMlpParams; e += blockDim.x) P[e] = params[e];
    __syncthreads();
    const int b = threadIdx.x;
    const int sidx = blockIdx.x * kTB + b;
    const bool valid = sidx < nb;
    float lsum = 0.0f;
    {
        float in[kMlpIn], h[kMlpH], g[kMlpH], y[kMlpOut];
        const int row = valid ? idx[sidx] : 0;
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) {
            in[k] = (X[(size_t)row * kMlpIn + k] - P[kOffMean + k]) * P[kOffIstd + k];
            a0[b * kMlpIn + k] = in[k];
        }
        mlp_layer<kMlpH, kMlpIn, true>(P + kOffW1, P + kOffB1, in, h);
        for (int k = 0; k < kMlpH; ++k) a1[b * kMlpH + k] = h[k];
        mlp_layer<kMlpH, kMlpH, true>(P + kOffW2, P + kOffB2, h, g);
        for (int k = 0; k < kMlpH; ++k) a2[b * kMlpH + k] = g[k];
        mlp_layer<kMlpH, kMlpH, true>(P + kOffW3, P + kOffB3, g, h);
        for (int k = 0; k < kMlpH; ++k) a3[b * kMlpH + k] = h[k];
        mlp_layer<kMlpOut, kMlpH, false>(P + kOffW4, P + kOffB4, h, y);
        for (int o = 0; o < kMlpOut; ++o) {
            const float r = valid ? (y[o] - Y[(size_t)row * kMlpOut + o]) : 0.0f;
            lsum += r * r;
            d4[b * kMlpOut + o] = 2.0f * r * inv_count;
        }
        // back through layers 4, 3, 2
        for (int k = 0; k < kMlpH; ++k) {
            float s = 0.0f;
            for (int o = 0; o < kMlpOut; ++o) s += P[kOffW4 + o * kMlpH + k] * d4[b * kMlpOut + o];
            d3[b * kMlpH + k] = a3[b * kMlpH + k] > 0.0f ? s : 0.0f;
        }
        for (int k = 0; k < kMlpH; ++k) {
            float s = 0.0f;
            for (int o = 0; o < kMlpH; ++o) s += P[kOffW3 + o * kMlpH + k] * d3[b * kMlpH + o];
            d2[b * kMlpH + k] = a2[b * kMlpH + k] > 0.0f ? s : 0.0f;
        }
        for (int k = 0; k < kMlpH; ++k) {
            float s = 0.0f;
            for (int o = 0; o < kMlpH; ++o) s += P[kOffW2 + o * kMlpH + k] * d2[b * kMlpH + o];
            d1[b * kMlpH + k] = a1[b * kMlpH + k] > 0.0f ? s : 0.0f;
        }
    }
    __syncthreads();
    // outer products summed over the block's samples
    auto outer = [&](const float* d, int dn, const float* a, int an, int offW, int offB) {
        for (int e = threadIdx.x; e < dn * an; e += blockDim.x) {
            const int o = e / an, k = e % an;
            float s = 0.0f;
            for (int q = 0; q < kTB; ++q) s += d[q * dn + o] * a[q * an + k];
            atomicAdd(&grad[offW + e], s);
        }
        for (int o = threadIdx.x; o < dn; o += blockDim.x) {
            float s = 0.0f;
            for (int q = 0; q < kTB; ++q) s += d[q * dn + o];
            atomicAdd(&grad[offB + o], s);
        }
    };
    outer(d4, kMlpOut, a3, kMlpH, kOffW4, kOffB4);
    outer(d3, kMlpH, a2, kMlpH, kOffW3, kOffB3);
    outer(d2, kMlpH, a1, kMlpH, kOffW2, kOffB2);
    outer(d1, kMlpH, a0, kMlpIn, kOffW1, kOffB1);
    for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, lsum);
}

__global__ void k_adam(int nparam, int first, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1t, float b2t) {
    const int k = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nparam) return;
    const float gk = g[k];
    const float mk = 0.9f * m[k] + 0.1f * gk;
    const float vk = 0.999f * v[k] + 0.001f * gk * gk;
    m[k] = mk;
    v[k] = vk;
    const float mh = mk / (1.0f - b1t), vh = vk / (1.0f - b2t);
    p[k] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

// Batched inference with the routine the list kernel uses: a warp per 32
// samples on the tensor cores (FP16 operands, FP32 accumulation).
__global__ void __launch_bounds__(128) k_mlp_infer(const float* __restrict__ params, const float* __restrict__ X,
                                                   int n, float* __restrict__ Y) {
    extern __shared__ __align__(16) float sm_inf[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* Xs = sm_inf + wib * kWarpTcFloats;
    float* Ys = Xs + 32 * kMlpInP;
    const float* S = params + kMlpInfOff;
    const int base = (blockIdx.x * blockDim.x) + wib * 32;
    const int cnt = max(0, min(32, n - base));
    if (cnt == 0) return;  // whole warp
    const int q = base + lane;
    if (lane < cnt) {
        float x[kMlpIn];
        for (int k = 0; k < kMlpIn; ++k) x[k] = X[(size_t)q * kMlpIn + k];
        mlp_input(S, x, Xs + lane * kMlpInP);
    }
    __syncwarp();
    warp_mlp_tc(params, Xs, Ys, cnt, lane);
    if (lane < cnt)
        for (int o = 0; o < kMlpOut; ++o) Y[(size_t)q * kMlpOut + o] = Ys[lane * kMlpOutP + o];
}

size_t infer_smem(int threads) { return sizeof(float) * (size_t)(threads / 32) * kWarpTcFloats; }

size_t train_smem() {
    return sizeof(float) * (kMlpParams + kTB * (kMlpIn + 3 * kMlpH + kMlpOut + 3 * kMlpH));
}

struct DevF {
    DevBuf b;
    float* p(size_t n) {
        if (b.ensure(sizeof(float) * std::max<size_t>(n, 1))) return nullptr;
        return b.as<float>();
    }
};

}  // namespace

int selector_node_norms(Workspace& ws, const TreeDev& t, int P, const double* d_sorted_damp, cudaStream_t st) {
    const int M = t.num_nodes;
    FMM_TRY(ws.sel_norms.ensure(sizeof(float) * (size_t)M * (P + 2)));
    count_launches(1);
    k_node_norms<<<grid_for(M, 128), 128, 0, st>>>(M, P, ws.wred.as<double>(), t, d_sorted_damp,
                                                   ws.sel_norms.as<float>(),
                                                   ws.sel_norms.as<float>() + (size_t)M * (P + 1));
    if (d_sorted_damp) {
        count_launches(1);
        k_dmin_up<<<grid_for(M, 128), 128, 0, st>>>(M, t, ws.sel_norms.as<float>() + (size_t)M * (P + 1));
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// Labels and features of sampled far pairs (device arrays).
int selector_pair_data(Workspace& ws, const Particles& Pt, const TreeDev& t, int P, const int2* d_pairs, int npairs,
                       float* d_feats, float* d_labels, cudaStream_t st) {
    const int m = dim_to_order(Pt.dim);
    const int M = t.num_nodes;
    const float* lnorm = ws.sel_norms.as<float>();
    const float* dmin = lnorm + (size_t)M * (P + 1);
    count_launches(1);
    k_pair_feats<<<grid_for(npairs, 128), 128, 0, st>>>(t, lnorm, dmin, P, d_pairs, npairs, d_feats);
    const int N = 2 * P, nTr = rbase_s(N + 1), nr = (P + 1) * (P + 1), nq = nT(P);
    const size_t per_warp = sizeof(double) * (2 * nTr + nr + nr + nq + kLabT * 3 + kLabT * 3 * 13 + (N + 1));
    const int wpb = 4;
    const size_t sm = per_warp * wpb;
    switch (m) {
        case 0:
            cudaFuncSetAttribute((const void*)k_pair_errors<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            count_launches(1);
            k_pair_errors<0><<<grid_for(npairs, wpb), 32 * wpb, sm, st>>>(
                t, P, d_pairs, npairs, ws.sx.as<double>(), ws.sy.as<double>(), ws.sz.as<double>(), ws.smc.as<double>(),
                Pt.n, ws.wred.as<double>(), d_labels);
            break;
        case 1:
            cudaFuncSetAttribute((const void*)k_pair_errors<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            count_launches(1);
            k_pair_errors<1><<<grid_for(npairs, wpb), 32 * wpb, sm, st>>>(
                t, P, d_pairs, npairs, ws.sx.as<double>(), ws.sy.as<double>(), ws.sz.as<double>(), ws.smc.as<double>(),
                Pt.n, ws.wred.as<double>(), d_labels);
            break;
        case 2:
            cudaFuncSetAttribute((const void*)k_pair_errors<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            count_launches(1);
            k_pair_errors<2><<<grid_for(npairs, wpb), 32 * wpb, sm, st>>>(
                t, P, d_pairs, npairs, ws.sx.as<double>(), ws.sy.as<double>(), ws.sz.as<double>(), ws.smc.as<double>(),
                Pt.n, ws.wred.as<double>(), d_labels);
            break;
        default:
            return FMM_ENOTSUP;
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int selector_unpack_far(Workspace& ws, const TreeDev& t, int2* d_out, cudaStream_t st) {
    if (t.nfar <= 0) return FMM_OK;
    count_launches(1);
    k_unpack_far<<<grid_for(t.nfar, 256), 256, 0, st>>>(t.nfar, ws.far_sorted.as<uint64_t>(), d_out);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

using namespace fmm;

extern "C" {

int fmm_mlp_param_count(void) { return kMlpParams; }
int fmm_selector_param_count(void) { return kMlpParams; }

// Training data of the selector for one system: features and log10 errors
// at orders 2..12 of up to max_pairs far pairs sampled uniformly from the
// far list of the reference acceptance test at `theta`.
int fmm_selector_collect(int64_t n, const double* X, int mdim, const double* mp, const double* damp, int ncrit,
                         double theta, int max_pairs, uint64_t seed, float* feats, float* labels, int* npairs_out,
                         int32_t* pairs_out) {
    if (n < 2 || !X || !mp || ncrit < 1 || !(theta > 0) || max_pairs < 1 || !feats || !labels || !npairs_out)
        return FMM_EINVAL;
    const int m = dim_to_order(mdim);
    if (m < 0 || m > 2) return FMM_ENOTSUP;
    const int P = kQmax;
    Workspace& ws = thread_workspace();
    cudaStream_t st = nullptr;
    FMM_TRY(ws.in_coords.ensure(sizeof(double) * 3 * n));
    FMM_TRY(ws.in_mp.ensure(sizeof(double) * (size_t)mdim * n));
    FMM_TRY(ws.in_damp.ensure(sizeof(double) * n));
    FMM_CUDA_TRY(cudaMemcpy(ws.in_coords.p, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(ws.in_mp.p, mp, sizeof(double) * (size_t)mdim * n, cudaMemcpyHostToDevice));
    if (damp) FMM_CUDA_TRY(cudaMemcpy(ws.in_damp.p, damp, sizeof(double) * n, cudaMemcpyHostToDevice));
    Particles Pt{n, ws.in_coords.as<double>(), mdim, ws.in_mp.as<double>(), 0, nullptr,
                 damp ? ws.in_damp.as<double>() : nullptr, DAMP_NONE};
    TreeParams tp{ncrit, theta, 1, 0, {0, 0, 0}, 0, 0.0, P};
    TreeDev t;
    FMM_TRY(build_tree(ws, Pt.x, n, tp, t, st));
    FMM_TRY(build_lists(ws, t, tp, st));
    FMM_TRY(gather_sorted(ws, Pt, t, st));
    FMM_TRY(launch_p2m_m2m(ws, Pt, t, P, st));
    FMM_TRY(launch_reduce_moments(ws, t, P, st));
    FMM_TRY(selector_node_norms(ws, t, P, damp ? ws.sd.as<double>() : nullptr, st));
    if (t.nfar < 1) {
        *npairs_out = 0;
        return FMM_OK;
    }
    // all far pairs to the host, a uniform sample back
    DevBuf all, sel, fd, ld;
    FMM_TRY(all.ensure(sizeof(int2) * (size_t)t.nfar));
    FMM_TRY(selector_unpack_far(ws, t, all.as<int2>(), st));
    std::vector<int2> hp((size_t)t.nfar);
    FMM_CUDA_TRY(cudaMemcpy(hp.data(), all.p, sizeof(int2) * t.nfar, cudaMemcpyDeviceToHost));
    std::mt19937_64 rng(seed);
    std::shuffle(hp.begin(), hp.end(), rng);
    const int np = (int)std::min<int64_t>(max_pairs, t.nfar);
    FMM_TRY(sel.ensure(sizeof(int2) * np));
    FMM_TRY(fd.ensure(sizeof(float) * (size_t)np * kMlpIn));
    FMM_TRY(ld.ensure(sizeof(float) * (size_t)np * kMlpOut));
    FMM_CUDA_TRY(cudaMemcpy(sel.p, hp.data(), sizeof(int2) * np, cudaMemcpyHostToDevice));
    if (pairs_out)
        for (int q = 0; q < np; ++q) {
            pairs_out[2 * q] = hp[q].x;
            pairs_out[2 * q + 1] = hp[q].y;
        }
    FMM_TRY(selector_pair_data(ws, Pt, t, P, sel.as<int2>(), np, fd.as<float>(), ld.as<float>(), st));
    FMM_CUDA_TRY(cudaMemcpy(feats, fd.p, sizeof(float) * (size_t)np * kMlpIn, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(labels, ld.p, sizeof(float) * (size_t)np * kMlpOut, cudaMemcpyDeviceToHost));
    *npairs_out = np;
    all.release();
    sel.release();
    fd.release();
    ld.release();
    return FMM_OK;
}

int fmm_mlp_forward(const float* params, const float* x, int64_t n, float* y) {
    if (!params || !x || !y || n < 1) return FMM_EINVAL;
    DevF P, X, Y;
    float* dp = P.p(kMlpBufFloats);  // blob, then its inference layout
    float* dx = X.p((size_t)n * kMlpIn);
    float* dy = Y.p((size_t)n * kMlpOut);
    if (!dp || !dx || !dy) return FMM_ENOMEM;
    FMM_CUDA_TRY(cudaMemcpy(dp, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(dx, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
    count_launches(1);
    k_mlp_stage_global<<<1, 256>>>(dp);
    FMM_CUDA_TRY(cudaFuncSetAttribute((const void*)k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)infer_smem(128)));
    count_launches(1);
    k_mlp_infer<<<grid_for(n, 128), 128, infer_smem(128)>>>(dp, dx, (int)n, dy);
    FMM_CUDA_TRY(cudaMemcpy(y, dy, sizeof(float) * n * kMlpOut, cudaMemcpyDeviceToHost));
    return FMM_OK;
}

// Gradient of the mean squared error over the n samples (mean over samples
// and outputs) with respect to the trainable parameters; grad has
// kMlpParams entries (the normalisation entries stay zero).  *loss receives
// the mean squared error.
int fmm_mlp_grad(const float* params, const float* x, const float* y, int64_t n, float* grad, float* loss) {
    if (!params || !x || !y || !grad || n < 1) return FMM_EINVAL;
    DevF P, X, Y, G, L, I;
    float* dp = P.p(kMlpParams);
    float* dx = X.p((size_t)n * kMlpIn);
    float* dy = Y.p((size_t)n * kMlpOut);
    float* dg = G.p(kMlpParams);
    float* dl = L.p(1);
    int* di = reinterpret_cast<int*>(I.p((size_t)n));
    if (!dp || !dx || !dy || !dg || !dl || !di) return FMM_ENOMEM;
    std::vector<int> idx((size_t)n);
    for (int64_t q = 0; q < n; ++q) idx[q] = (int)q;
    FMM_CUDA_TRY(cudaMemcpy(dp, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(dx, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(dy, y, sizeof(float) * n * kMlpOut, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(di, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemset(dg, 0, sizeof(float) * kMlpParams));
    FMM_CUDA_TRY(cudaMemset(dl, 0, sizeof(float)));
    const size_t sm = train_smem();
    FMM_CUDA_TRY(cudaFuncSetAttribute((const void*)k_mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    count_launches(1);
    k_mlp_fwd_bwd<<<grid_for(n, kTB), kTB, sm>>>(dp, dx, dy, di, (int)n, 1.0f / (float)(n * kMlpOut), dg, dl);
    FMM_CUDA_TRY(cudaMemcpy(grad, dg, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    float ls = 0;
    FMM_CUDA_TRY(cudaMemcpy(&ls, dl, sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) *loss = ls / (float)(n * kMlpOut);
    return FMM_OK;
}

// Adam training of the parameters (in/out) on n samples; the normalisation
// entries of `params` must already be set.  losses[e] receives the mean
// squared error of epoch e (before the epoch's updates were complete).
int fmm_mlp_train(float* params, const float* x, const float* y, int64_t n, int epochs, int batch, float lr,
                  uint64_t seed, float* losses) {
    if (!params || !x || !y || n < kTB || epochs < 1 || batch < kTB) return FMM_EINVAL;
    DevF P, X, Y, G, Mm, Vv, L, I;
    float* dp = P.p(kMlpParams);
    float* dx = X.p((size_t)n * kMlpIn);
    float* dy = Y.p((size_t)n * kMlpOut);
    float* dg = G.p(kMlpParams);
    float* dm = Mm.p(kMlpParams);
    float* dv = Vv.p(kMlpParams);
    float* dl = L.p(1);
    int* di = reinterpret_cast<int*>(I.p((size_t)n));
    if (!dp || !dx || !dy || !dg || !dm || !dv || !dl || !di) return FMM_ENOMEM;
    FMM_CUDA_TRY(cudaMemcpy(dp, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(dx, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(dy, y, sizeof(float) * n * kMlpOut, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemset(dm, 0, sizeof(float) * kMlpParams));
    FMM_CUDA_TRY(cudaMemset(dv, 0, sizeof(float) * kMlpParams));
    const size_t sm = train_smem();
    FMM_CUDA_TRY(cudaFuncSetAttribute((const void*)k_mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    std::vector<int> idx((size_t)n);
    std::mt19937_64 rng(seed);
    float b1t = 1.0f, b2t = 1.0f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int64_t q = 0; q < n; ++q) idx[q] = (int)q;
        std::shuffle(idx.begin(), idx.end(), rng);
        FMM_CUDA_TRY(cudaMemcpy(di, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
        FMM_CUDA_TRY(cudaMemset(dl, 0, sizeof(float)));
        const float lr_e = lr * (ep < epochs / 2 ? 1.0f : (ep < 3 * epochs / 4 ? 0.3f : 0.1f));
        for (int64_t b0 = 0; b0 + batch <= n; b0 += batch) {
            FMM_CUDA_TRY(cudaMemsetAsync(dg, 0, sizeof(float) * kMlpParams));
            count_launches(1);
            k_mlp_fwd_bwd<<<batch / kTB, kTB, sm>>>(dp, dx, dy, di + b0, batch, 1.0f / (float)(batch * kMlpOut), dg,
                                                    dl);
            b1t *= 0.9f;
            b2t *= 0.999f;
            count_launches(1);
            k_adam<<<grid_for(kMlpParams - kOffW1, 256), 256>>>(kMlpParams, kOffW1, dp, dg, dm, dv, lr_e, b1t, b2t);
        }
        float ls = 0;
        FMM_CUDA_TRY(cudaMemcpy(&ls, dl, sizeof(float), cudaMemcpyDeviceToHost));
        if (losses) losses[ep] = ls / (float)((n / batch) * batch * kMlpOut);
    }
    FMM_CUDA_TRY(cudaMemcpy(params, dp, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // extern "C"

// P2M, M2M, L2L and L2P (reference: src/fmm.F90:387-546 and 981-1132).
//
// Cell multipoles are kept scaled, M'_t = M_t / t! (t! = tx! ty! tz!), so
// every translation is a convolution with the scaled powers d^u / u!:
//   P2M  M'_t(leaf)   = sum_i sum_{s<=t} (d_i^(t-s)/(t-s)!) M'_s(i)
//   M2M  M'_t(parent) = sum_c sum_{u<=t} (d_c^u/u!) M'_{t-u}(c)
//   L2L  L_t(child)  += sum_u L_{t+u}(parent) d^u/u!
//   L2P  F_t(i)      += sum_u L_{t+u}(leaf) d_i^u/u!,  |t| <= f
// (the reference shifts each leaf straight into every ancestor; level by
// level is the same sum since the shifts compose exactly).
//
// P2M runs a block per leaf with the particles' moments times their scaled
// powers accumulated per power u in registers; M2M and L2L a block per parent
// node, each as three one-dimensional shifts of a dense expansion; L2P a work
// item per (particle, output) with the local expansion evaluated by nested
// Horner schemes in the leaf's length unit (FP32 in the mixed-precision path,
// where the local expansion's terms decrease with order and carry no
// cancellation between per-atom terms), its coefficients staged from a table
// built once per (p, f).
// P2M, M2M and L2L are FP64 in the plain path and double-float (FP32 pipe,
// exact products by FMA, ~48-bit sums) in the mixed path, M2M and L2L with
// an FP64 fallback for blocks whose powers or moments leave the range where
// FP32 exponents suffice.
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"
#include "pair_x2.cuh"

namespace fmm {

namespace {

__host__ __device__ constexpr int pack3(int x, int y, int z) { return x | (y << 8) | (z << 16); }
__device__ __forceinline__ int ux_(int c) { return c & 0xff; }
__device__ __forceinline__ int uy_(int c) { return (c >> 8) & 0xff; }
__device__ __forceinline__ int uz_(int c) { return (c >> 16) & 0xff; }

// Packed components (x | y << 8 | z << 16) of order <= p: in the packed
// order, then sorted by z, by y and by x (the orders in which the M2M's
// three shifts visit their outputs, so that the outputs of a warp have the
// same number of terms), uploaded once per order.
struct TabView {
    int nq, comp, byz, byy, byx;
};

int hidx(int x, int y, int z) { return nT(x + y + z - 1) + ((y + z) * (y + z + 1)) / 2 + z; }

int ensure_tables(Workspace& ws, int p, TabView* out, cudaStream_t st) {
    const int nq = nT(p);
    out->nq = nq;
    out->comp = 0;
    out->byz = nq;
    out->byy = 2 * nq;
    out->byx = 3 * nq;
    if (ws.xlate_p == p) return FMM_OK;
    std::vector<int> comp;
    for (int k = 0; k <= p; ++k)
        for (int x = k; x >= 0; --x)
            for (int y = k - x; y >= 0; --y) comp.push_back(pack3(x, y, k - x - y));
    std::vector<int> all(comp);
    for (int sh : {16, 8, 0}) {  // by z, by y, by x
        std::vector<int> o(comp);
        std::stable_sort(o.begin(), o.end(), [sh](int a, int b) { return ((a >> sh) & 0xff) < ((b >> sh) & 0xff); });
        all.insert(all.end(), o.begin(), o.end());
    }
    FMM_TRY(ws.xlate.ensure(sizeof(int) * all.size()));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.xlate.p, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    ws.xlate_p = p;
    return FMM_OK;
}

// L2P coefficients of the outputs t (|t| <= f), each in Horner order (ux,
// uy, uz descending, |u| <= p - |t|): segment starts seg[nT(f)+1], then per
// coefficient the index of L_{t+u} and its order (w | k << 16), then (from an
// 8-byte boundary) 1 / (ux! uy! uz!) as FP64.  Once per (p, f).
struct L2pTab {
    int nf, ncoef, seg, wk, fac;  // offsets in ints
};

int ensure_l2p_table(Workspace& ws, int p, int f, L2pTab* out, cudaStream_t st) {
    const int nf = nT(f);
    std::vector<int> seg(1, 0), wk;
    std::vector<double> fac;
    for (int k = 0, tq = 0; k <= f; ++k)
        for (int tx = k; tx >= 0; --tx)
            for (int ty = k - tx; ty >= 0; --ty, ++tq) {
                const int tz = k - tx - ty, rem = p - k;
                for (int ux = rem; ux >= 0; --ux)
                    for (int uy = rem - ux; uy >= 0; --uy)
                        for (int uz = rem - ux - uy; uz >= 0; --uz) {
                            wk.push_back(hidx(tx + ux, ty + uy, tz + uz) | ((k + ux + uy + uz) << 16));
                            fac.push_back(1.0 / (cfact(ux) * cfact(uy) * cfact(uz)));
                        }
                seg.push_back((int)wk.size());
            }
    L2pTab v;
    v.nf = nf;
    v.ncoef = (int)wk.size();
    v.seg = 0;
    v.wk = nf + 1;
    v.fac = (v.wk + v.ncoef + 1) & ~1;
    *out = v;
    if (ws.l2pt_p == p && ws.l2pt_f == f) return FMM_OK;
    std::vector<int> all((size_t)v.fac + 2 * (size_t)v.ncoef, 0);
    std::copy(seg.begin(), seg.end(), all.begin() + v.seg);
    std::copy(wk.begin(), wk.end(), all.begin() + v.wk);
    std::memcpy(all.data() + v.fac, fac.data(), sizeof(double) * fac.size());
    FMM_TRY(ws.l2pt.ensure(sizeof(int) * all.size()));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.l2pt.p, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    ws.l2pt_p = p;
    ws.l2pt_f = f;
    return FMM_OK;
}

__device__ __forceinline__ void copy_ints(int* dst, const int* __restrict__ src, int n) {
    for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = src[e];
}

// 1/a for a = 0..2 kMaxP + 1 (no divisions on the FP64 pipe)
__constant__ double cInvInt[2 * kMaxP + 2] = {
#define FMM_X(a) ((a) == 0 ? 0.0 : 1.0 / (a)),
    FMM_X(0) FMM_X(1) FMM_X(2) FMM_X(3) FMM_X(4) FMM_X(5) FMM_X(6) FMM_X(7) FMM_X(8) FMM_X(9) FMM_X(10) FMM_X(11)
    FMM_X(12) FMM_X(13) FMM_X(14) FMM_X(15) FMM_X(16) FMM_X(17) FMM_X(18) FMM_X(19) FMM_X(20) FMM_X(21) FMM_X(22)
    FMM_X(23) FMM_X(24) FMM_X(25)
#undef FMM_X
};
static_assert(kMaxP == 12, "the inverse table covers orders up to 12");
// 1/a as double-float pairs, a = 0..kMaxP
__constant__ float2 cInvIntF[kMaxP + 1] = {
#define FMM_XF(a) {(a) == 0 ? 0.0f : (float)(1.0 / (a)), (a) == 0 ? 0.0f : (float)(1.0 / (a) - (double)(float)(1.0 / (a)))},
    FMM_XF(0) FMM_XF(1) FMM_XF(2) FMM_XF(3) FMM_XF(4) FMM_XF(5) FMM_XF(6) FMM_XF(7) FMM_XF(8) FMM_XF(9) FMM_XF(10)
    FMM_XF(11) FMM_XF(12)
#undef FMM_XF
};

// e[a] = d^a / a!, a = 0..p
__device__ __forceinline__ void scaled_powers(double d, int p, double* e) {
    e[0] = 1.0;
    for (int a = 1; a <= p; ++a) e[a] = e[a - 1] * d * cInvInt[a];
}

// Product of two double-float pairs (hi, lo), renormalised.
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float s = p + e;
    return make_float2(s, e - (s - p));
}

// a += x * y in double-float (exact product by FMA, TwoSum accumulation).
__device__ __forceinline__ void df_mac(float2 x, float2 y, float& h, float& l) {
    const float pr = x.x * y.x;
    float er = fmaf(x.x, y.x, -pr);
    er = fmaf(x.x, y.y, er);
    er = fmaf(x.y, y.x, er);
    const float sum = h + pr;
    const float bb = sum - h;
    l += ((h - (sum - bb)) + (pr - bb)) + er;
    h = sum;
}

// (hi, lo) FP32 pair of an FP64 value from its bit pattern alone (no FP64
// instruction): hi the value truncated to 24 significant bits, lo the
// remaining 29 bits rounded to FP32.  Zero, magnitudes outside the normal
// FP32 range and non-finite values take the FP64 conversion.
__device__ __forceinline__ float2 split_bits(double w) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(w);
    if ((b << 1) == 0ull) return make_float2(0.0f, 0.0f);
    const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
    const int e = (int)((hi32 >> 20) & 0x7ffu);
    if (e < 1023 - 126 || e > 1023 + 127) {
        const float h = (float)w;
        return make_float2(h, (float)(w - (double)h));
    }
    const unsigned sgn = hi32 & 0x80000000u;
    const float h = __uint_as_float(sgn | ((unsigned)(e - 1023 + 127) << 23) | ((hi32 & 0xfffffu) << 3) | (lo32 >> 29));
    // the low 29 bits weigh 2^(e - 1075); below 2^-126 that weight is applied
    // in two steps (e >= 897 keeps the first step's exponent positive)
    const int se = e - 1075 + 127;
    const float r = __uint2float_rn(lo32 & 0x1fffffffu);
    const float l = se > 0 ? r * __uint_as_float((unsigned)se << 23)
                           : (r * __uint_as_float((unsigned)(se + 64) << 23)) * 0x1p-64f;
    return make_float2(h, sgn ? -l : l);
}

// split_bits, and *big set for magnitudes from 2^99 up or non-finite values
// (outside the range where double-float products keep their precision),
// on integer instructions.
__device__ __forceinline__ float2 to_df_bits(double w, int* big) {
    const int e = (int)(((unsigned long long)__double_as_longlong(w) >> 52) & 0x7ffu);
    if (e >= 1023 + 99) *big = 1;
    return split_bits(w);
}

// Arithmetic of the shifts: FP64, or double-float pairs on the FP32 pipe.
template <bool DF>
struct XOps;
template <>
struct XOps<false> {
    using V = double;
    struct Acc {
        double a = 0.0;
        __device__ __forceinline__ void mac(double x, double y) { a = fma(x, y, a); }
        __device__ __forceinline__ void add(double x) { a += x; }
        __device__ __forceinline__ double val() const { return a; }
    };
    static __device__ __forceinline__ double in(double w, int*) { return w; }
    static __device__ __forceinline__ double mul(double x, double y) { return x * y; }
    static __device__ __forceinline__ double split(double w) { return w; }
    static __device__ __forceinline__ double neg(double x) { return -x; }
    static __device__ __forceinline__ double one() { return 1.0; }
    static __device__ __forceinline__ double inv_int(int a) { return cInvInt[a]; }
    static __device__ __forceinline__ double out(double v) { return v; }
};
template <>
struct XOps<true> {
    using V = float2;
    struct Acc {
        float h = 0.0f, l = 0.0f;
        __device__ __forceinline__ void mac(float2 x, float2 y) { df_mac(x, y, h, l); }
        __device__ __forceinline__ void add(float2 x) {
            const float sum = h + x.x;
            const float bb = sum - h;
            l += ((h - (sum - bb)) + (x.x - bb)) + x.y;
            h = sum;
        }
        __device__ __forceinline__ float2 val() const {
            const float s = h + l;
            return make_float2(s, l - (s - h));
        }
    };
    static __device__ __forceinline__ float2 in(double w, int* big) { return to_df_bits(w, big); }
    static __device__ __forceinline__ float2 mul(float2 x, float2 y) { return df_mul(x, y); }
    static __device__ __forceinline__ float2 split(double w) { return split_bits(w); }
    static __device__ __forceinline__ float2 neg(float2 x) { return make_float2(-x.x, -x.y); }
    static __device__ __forceinline__ float2 one() { return make_float2(1.0f, 0.0f); }
    static __device__ __forceinline__ float2 inv_int(int a) { return cInvIntF[a]; }
    static __device__ __forceinline__ double out(float2 v) { return (double)v.x + (double)v.y; }
};

// ---------------------------------------------------------------- P2M
// Block per leaf.  With dp_i[u] = d_i^u / u! (d_i = x_i - c_leaf) the leaf's
// moments are M'_t = sum_{s <= t} A_s[t - s], A_s[u] = sum_i M'_s(i) dp_i[u]
// (|s| <= m, |u| <= p - |s|): a product of the particles' moments (NM per
// particle) and powers, accumulated by the thread that owns u in registers
// (NM independent accumulators per u, the moments read as shared-memory
// broadcasts, dp_i[u] formed in registers from the particle's powers per
// axis), then the short sums over s.
constexpr int kP2mBatch = 64;

// Shared-memory entries (8 bytes) of the P2M staging area: one batch's
// powers and moments, or the leaf's A_s[u] at the end.
__host__ __device__ __forceinline__ int p2m_stage_entries(int p, int nm) {
    const int a = kP2mBatch * (3 * (p + 1) + nm + 1), b = nT(p) * nm;
    return a > b ? a : b;
}

// Two double-float multiply-adds at once in packed FP32 (f32x2): the
// accumulators (h, l) of moments s and s' as packed pairs H, L, the product
// x * (y_s, y_s'), with x = (xh, xl) broadcast (nxh = -xh) and y given as
// packed hi and lo parts.  Each half is df_mac's exact sequence (the
// product's rounding error by FMA, TwoSum into h), written with -pr.
__device__ __forceinline__ void df_mac_x2(f2 xh, f2 nxh, f2 xl, f2 yh, f2 yl, f2& H, f2& L) {
    const f2 npr = nxh * yh;
    f2 er = fma2(xh, yh, npr);
    er = fma2(xh, yl, er);
    er = fma2(xl, yh, er);
    const f2 sum = H - npr;
    const f2 bb = sum - H;
    L = L + (((H - (sum - bb)) - (npr + bb)) + er);
    H = sum;
}

__device__ __forceinline__ int pk_index(int x, int y, int z) {
    const int k = x + y + z, yz = y + z;
    return k * (k + 1) * (k + 2) / 6 + yz * (yz + 1) / 2 + z;
}

template <bool DF, int NM, int KS, int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_p2m(const TreeDev t, const double* __restrict__ sx,
                                                      const double* __restrict__ sy, const double* __restrict__ sz,
                                                      const double* __restrict__ smc, int64_t n, int p,
                                                      const int* __restrict__ tab, TabView v,
                                                      double* __restrict__ mom) {
    using O = XOps<DF>;
    using V = typename O::V;
    constexpr int KB = kP2mBatch;
    extern __shared__ __align__(16) double sm_p2m[];
    const int nq = v.nq, P1 = p + 1;
    V* stage = reinterpret_cast<V*>(sm_p2m);  // [KB][3][p+1] powers per axis, [KB][NM] moments
    V* A = stage;                             // [nq][NM], after the last batch
    int* comp = reinterpret_cast<int*>(stage + p2m_stage_entries(p, NM));
    copy_ints(comp, tab + v.comp, nq);
    const int leaf = t.leaves[blockIdx.x];
    const double cx = t.cx[leaf], cy = t.cy[leaf], cz = t.cz[leaf];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    __syncthreads();
    // this thread's u (KS slots) and the moments s that pair with each
    int ux[KS], uy[KS], uz[KS], ns[KS];
#pragma unroll
    for (int r = 0; r < KS; ++r) {
        const int u = threadIdx.x + NT * r;
        ns[r] = 0;
        ux[r] = uy[r] = uz[r] = 0;
        if (u < nq) {
            const int c = comp[u];
            ux[r] = ux_(c);
            uy[r] = uy_(c);
            uz[r] = uz_(c);
            const int rem = p - ux[r] - uy[r] - uz[r];
            ns[r] = min(NM, nT(rem));  // moments of orders <= rem
        }
    }
    typename O::Acc acc[KS][DF ? 1 : NM];
    // double-float path: the accumulators of moments (2k, 2k + 1) as packed pairs
    f2 PH[KS][DF ? (NM + 1) / 2 : 1], PL[KS][DF ? (NM + 1) / 2 : 1];
    if constexpr (DF) {
#pragma unroll
        for (int r = 0; r < KS; ++r)
#pragma unroll
            for (int k = 0; k < (NM + 1) / 2; ++k) PH[r][k] = PL[r][k] = bc2(0.0f);
    }
    for (int b0 = 0; b0 < cnt; b0 += KB) {
        const int nb = min(KB, cnt - b0);
        // scaled powers d^a / a! per particle axis and the moments M_s / s!
        // (sign of the potential convention), all of the batch at once
        for (int k = threadIdx.x; k < 3 * nb; k += NT) {
            const int b = k / 3, ax = k - 3 * b, i = s0 + b0 + b;
            const V d = O::split(ax == 0 ? sx[i] - cx : (ax == 1 ? sy[i] - cy : sz[i] - cz));
            V w = O::one();
            V* eb = stage + k * P1;
            eb[0] = w;
            for (int a = 1; a <= p; ++a) {
                w = O::mul(O::mul(w, d), O::inv_int(a));
                eb[a] = w;
            }
        }
        V* msb = stage + KB * 3 * P1;
        if constexpr (DF) {
            // moments in pairs (s, s + 1) as float4 (hi_s, hi_s+1, lo_s, lo_s+1)
            // (16-byte aligned: KB * 3 * P1 8-byte entries is even)
            constexpr int NMP = (NM + 1) / 2;
            float* mf = reinterpret_cast<float*>(msb);
            for (int idx = threadIdx.x; idx < nb * 2 * NMP; idx += NT) {
                const int b = idx / (2 * NMP), sidx = idx - b * (2 * NMP);
                V w = sidx < NM ? O::split(smc[(size_t)sidx * n + s0 + b0 + b]) : O::split(0.0);
                if (sidx < NM && ((order_of(sidx) + 1) % 2)) w = O::neg(w);
                float* e = mf + ((size_t)b * NMP + (sidx >> 1)) * 4 + (sidx & 1);
                e[0] = w.x;
                e[2] = w.y;
            }
        } else {
            for (int idx = threadIdx.x; idx < nb * NM; idx += NT) {
                const int b = idx / NM, sidx = idx - b * NM;
                const V w = O::split(smc[(size_t)sidx * n + s0 + b0 + b]);
                msb[idx] = ((order_of(sidx) + 1) % 2) ? O::neg(w) : w;
            }
        }
        __syncthreads();
        if constexpr (DF) {
            constexpr int NMP = (NM + 1) / 2;
            const float4* mq = reinterpret_cast<const float4*>(msb);
            for (int b = 0; b < nb; ++b) {
                const V* eb = stage + b * 3 * P1;
                f2 mh[NMP], ml[NMP];
#pragma unroll
                for (int k = 0; k < NMP; ++k) {
                    const float4 w = mq[(size_t)b * NMP + k];
                    mh[k] = mk2(w.x, w.y);
                    ml[k] = mk2(w.z, w.w);
                }
#pragma unroll
                for (int r = 0; r < KS; ++r) {
                    if (ns[r] == 0) continue;
                    const V dp = O::mul(O::mul(eb[ux[r]], eb[P1 + uy[r]]), eb[2 * P1 + uz[r]]);
                    const f2 xh = bc2(dp.x), nxh = bc2(-dp.x), xl = bc2(dp.y);
                    if (ns[r] == NM) {  // every moment (u of order <= p - m)
#pragma unroll
                        for (int k = 0; k < NMP; ++k) df_mac_x2(xh, nxh, xl, mh[k], ml[k], PH[r][k], PL[r][k]);
                    } else {
                        // pairs holding a moment below ns (the other half of
                        // the last pair feeds an accumulator that is not read)
#pragma unroll
                        for (int k = 0; k < NMP; ++k)
                            if (2 * k < ns[r]) df_mac_x2(xh, nxh, xl, mh[k], ml[k], PH[r][k], PL[r][k]);
                    }
                }
            }
        } else
        for (int b = 0; b < nb; ++b) {
            const V* eb = stage + b * 3 * P1;
            const V* mb = msb + b * NM;
            V m[NM];
#pragma unroll
            for (int sidx = 0; sidx < NM; ++sidx) m[sidx] = mb[sidx];
#pragma unroll
            for (int r = 0; r < KS; ++r) {
                if (ns[r] == 0) continue;
                const V dp = O::mul(O::mul(eb[ux[r]], eb[P1 + uy[r]]), eb[2 * P1 + uz[r]]);
                if (ns[r] == NM) {  // every moment (u of order <= p - m)
#pragma unroll
                    for (int sidx = 0; sidx < NM; ++sidx) acc[r][sidx].mac(dp, m[sidx]);
                } else {
#pragma unroll
                    for (int sidx = 0; sidx < NM; ++sidx)
                        if (sidx < ns[r]) acc[r][sidx].mac(dp, m[sidx]);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < KS; ++r) {
        const int u = threadIdx.x + NT * r;
#pragma unroll
        for (int sidx = 0; sidx < NM; ++sidx) {
            if (sidx >= ns[r]) continue;
            if constexpr (DF) {
                float h0, h1, l0, l1;
                sp2(PH[r][sidx >> 1], h0, h1);
                sp2(PL[r][sidx >> 1], l0, l1);
                typename O::Acc a;
                a.h = (sidx & 1) ? h1 : h0;
                a.l = (sidx & 1) ? l1 : l0;
                A[u * NM + sidx] = a.val();
            } else {
                A[u * NM + sidx] = acc[r][sidx].val();
            }
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nq; q += NT) {
        const int c = comp[q], tx = ux_(c), ty = uy_(c), tz = uz_(c);
        typename O::Acc sum;
#pragma unroll
        for (int sidx = 0; sidx < NM; ++sidx) {
            const int sc = comp[sidx], qx = ux_(sc), qy = uy_(sc), qz = uz_(sc);
            if (qx <= tx && qy <= ty && qz <= tz) sum.add(A[pk_index(tx - qx, ty - qy, tz - qz) * NM + sidx]);
        }
        mom[(size_t)leaf * nq + q] = O::out(sum.val());
    }
}

// ---------------------------------------------------------------- M2M / L2L
// Both translations factor over the axes, d^u / u! = (dx^ux/ux!)
// (dy^uy/uy!) (dz^uz/uz!), so each is three one-dimensional shifts (z, then
// y, then x) of an expansion held densely in shared memory, index
// (a (p+1) + b) (p+1) + c for the component (a, b, c): C(p+4,4) terms per
// shift instead of the C(p+6,6) of the direct sum, and no output of a shift
// has more than p+1 terms, so the block's outputs finish together.  A block
// per parent node takes its children one after another.
constexpr int kXThreads = 512;  // one output per thread up to order 12: a shift waits for at most p+1 terms
constexpr int kXOut = (nT(kMaxP) + kXThreads - 1) / kXThreads;  // outputs per thread

__device__ __forceinline__ int d3(int a, int b, int c, int P1) { return (a * P1 + b) * P1 + c; }

// Children of a node (ch[0..7], count in ch[8]) and the scaled powers
// d^a / a! of their offsets d = c_child - c_node, e[(k * 3 + axis) * (p+1) + a].
__device__ __forceinline__ void child_offsets(const TreeDev& t, int node, int p, int* ch, double* e) {
    if (threadIdx.x == 0) {
        int k = 0;
        for (int o = 0; o < 8; ++o) {
            const int c = t.child[8 * node + o];
            if (c >= 0) ch[k++] = c;
        }
        ch[8] = k;
    }
    __syncthreads();
    const int P1 = p + 1;
    if (threadIdx.x < 3 * ch[8]) {
        const int b = threadIdx.x / 3, ax = threadIdx.x % 3, c = ch[b];
        const double d = ax == 0 ? t.cx[c] - t.cx[node] : (ax == 1 ? t.cy[c] - t.cy[node] : t.cz[c] - t.cz[node]);
        scaled_powers(d, p, e + (b * 3 + ax) * P1);
    }
    __syncthreads();
}

// M2M of one parent: M'_t = sum_children sum_{u <= t} (d^u/u!) M'_{t-u}(child)
// as shifts along z (Y from X), y (X from Y) and x (into the accumulator of
// the thread's output), each visiting its outputs sorted by the number of
// terms; the next child's moments are loaded during the current child's
// shifts.  Writes the result unless *big was raised.
template <bool DF>
__device__ __forceinline__ void m2m_node(int node, int p, int nq, const int* comp, const int* byz, const int* byy,
                                         const int* byx, const int* ch, const double* e, void* buf, int* big,
                                         double* __restrict__ mom) {
    static_assert(kXOut == 1, "one output per thread");
    using O = XOps<DF>;
    using V = typename O::V;
    const int P1 = p + 1, n3 = P1 * P1 * P1, q = threadIdx.x;
    V* X = reinterpret_cast<V*>(buf);
    V* Y = X + n3;
    V* E = Y + n3;  // [8][3][p+1]
    const int nch = ch[8];
    for (int k = threadIdx.x; k < nch * 3 * P1; k += blockDim.x) E[k] = O::in(e[k], big);
    int cz = 0, cy = 0, cx = 0, xo = 0;
    if (q < nq) {
        cz = byz[q];
        cy = byy[q];
        cx = byx[q];
        xo = pk_index(cx & 0xff, (cx >> 8) & 0xff, cx >> 16);
    }
    double mnext = (q < nq && nch > 0) ? mom[(size_t)ch[0] * nq + q] : 0.0;
    typename O::Acc acc;
    for (int b = 0; b < nch; ++b) {
        if (q < nq) {
            const int cc = comp[q];
            X[d3(cc & 0xff, (cc >> 8) & 0xff, cc >> 16, P1)] = O::in(mnext, big);
        }
        __syncthreads();
        if (b + 1 < nch && q < nq) mnext = mom[(size_t)ch[b + 1] * nq + q];  // in flight during the shifts
        const V* ex = E + b * 3 * P1;
        const V* ey = ex + P1;
        const V* ez = ey + P1;
        if (q < nq) {
            const int x = cz & 0xff, y = (cz >> 8) & 0xff, z = cz >> 16;
            typename O::Acc s;
            for (int u = 0; u <= z; ++u) s.mac(ez[u], X[d3(x, y, z - u, P1)]);
            Y[d3(x, y, z, P1)] = s.val();
        }
        __syncthreads();
        if (q < nq) {
            const int x = cy & 0xff, y = (cy >> 8) & 0xff, z = cy >> 16;
            typename O::Acc s;
            for (int u = 0; u <= y; ++u) s.mac(ey[u], Y[d3(x, y - u, z, P1)]);
            X[d3(x, y, z, P1)] = s.val();
        }
        __syncthreads();
        if (q < nq) {
            const int x = cx & 0xff, y = (cx >> 8) & 0xff, z = cx >> 16;
            for (int u = 0; u <= x; ++u) acc.mac(ex[u], X[d3(x - u, y, z, P1)]);
        }
        __syncthreads();  // X is the next child's
    }
    if (DF && *big) return;
    if (q < nq) mom[(size_t)node * nq + xo] = O::out(acc.val());
}

// DF: double-float shifts, FP64 again for the blocks whose powers or moments
// leave the range where FP32 exponents suffice.
template <bool DF>
__global__ void __launch_bounds__(kXThreads) k_m2m(const TreeDev t, const int32_t* __restrict__ nodes, int p,
                                                   const int* __restrict__ tab, TabView v, double* __restrict__ mom) {
    extern __shared__ __align__(16) double sm_m2m[];
    __shared__ int big, ch[9];
    const int nq = v.nq, P1 = p + 1;
    const int node = nodes[blockIdx.x];
    if (t.is_leaf[node]) return;
    double* e = sm_m2m;                                          // [8][3][p+1]
    int* comp = reinterpret_cast<int*>(e + 8 * 3 * P1);          // [4][nq]: packed, by z, by y, by x
    void* buf = e + 8 * 3 * P1 + (4 * nq + 1) / 2;               // X, Y, E
    copy_ints(comp, tab + v.comp, 4 * nq);
    if (threadIdx.x == 0) big = 0;
    child_offsets(t, node, p, ch, e);
    m2m_node<DF>(node, p, nq, comp, comp + nq, comp + 2 * nq, comp + 3 * nq, ch, e, buf, &big, mom);
    if (DF) {
        __syncthreads();
        if (big) m2m_node<false>(node, p, nq, comp, comp + nq, comp + 2 * nq, comp + 3 * nq, ch, e, buf, &big, mom);
    }
}

// L2L of one parent into each child: L_t(child) += sum_u L_{t+u}(parent)
// d^u/u! (|t + u| <= p) as shifts along z (Y from X, the parent's
// expansion), y (Z from Y) and x (into the child's expansion).
template <bool DF>
__device__ __forceinline__ void l2l_node(int node, int p, int nq, const int* comp, const int* ch, const double* e,
                                         void* buf, int* big, double* __restrict__ loc) {
    static_assert(kXOut == 1, "one output per thread");
    using O = XOps<DF>;
    using V = typename O::V;
    const int P1 = p + 1, n3 = P1 * P1 * P1;
    V* X = reinterpret_cast<V*>(buf);
    V* Y = X + n3;
    V* Z = Y + n3;
    V* E = Z + n3;  // [8][3][p+1]
    const int nch = ch[8];
    for (int k = threadIdx.x; k < nch * 3 * P1; k += blockDim.x) E[k] = O::in(e[k], big);
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        const int cc = comp[q];
        X[d3(cc & 0xff, (cc >> 8) & 0xff, cc >> 16, P1)] = O::in(loc[(size_t)node * nq + q], big);
    }
    __syncthreads();
    if (DF && *big) return;  // every thread sees the flag after the barrier
    for (int b = 0; b < nch; ++b) {
        const V* ex = E + b * 3 * P1;
        const V* ey = ex + P1;
        const V* ez = ey + P1;
        // the child's own expansion, in flight during the shifts
        double* lc = loc + (size_t)ch[b] * nq;
        const double lprev = threadIdx.x < nq ? lc[threadIdx.x] : 0.0;
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int cc = comp[q], x = cc & 0xff, y = (cc >> 8) & 0xff, z = cc >> 16;
            typename O::Acc s;
            for (int u = 0; u <= p - x - y - z; ++u) s.mac(ez[u], X[d3(x, y, z + u, P1)]);
            Y[d3(x, y, z, P1)] = s.val();
        }
        __syncthreads();
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int cc = comp[q], x = cc & 0xff, y = (cc >> 8) & 0xff, z = cc >> 16;
            typename O::Acc s;
            for (int u = 0; u <= p - x - y - z; ++u) s.mac(ey[u], Y[d3(x, y + u, z, P1)]);
            Z[d3(x, y, z, P1)] = s.val();
        }
        __syncthreads();
        if (threadIdx.x < nq) {  // one output per thread
            const int q = threadIdx.x, cc = comp[q], x = cc & 0xff, y = (cc >> 8) & 0xff, z = cc >> 16;
            typename O::Acc s;
            for (int u = 0; u <= p - x - y - z; ++u) s.mac(ex[u], Z[d3(x + u, y, z, P1)]);
            lc[q] = lprev + O::out(s.val());
        }
        __syncthreads();  // Y and Z are the next child's
    }
}

template <bool DF>
__global__ void __launch_bounds__(kXThreads) k_l2l(const TreeDev t, const int32_t* __restrict__ nodes, int p,
                                                   const int* __restrict__ tab, TabView v, double* __restrict__ loc) {
    extern __shared__ __align__(16) double sm_l2l[];
    __shared__ int big, ch[9];
    const int nq = v.nq, P1 = p + 1;
    const int node = nodes[blockIdx.x];
    if (t.is_leaf[node]) return;
    double* e = sm_l2l;                                          // [8][3][p+1]
    int* comp = reinterpret_cast<int*>(e + 8 * 3 * P1);          // [nq]
    void* buf = e + 8 * 3 * P1 + (nq + 1) / 2;                   // X, Y, Z, E
    copy_ints(comp, tab + v.comp, nq);
    if (threadIdx.x == 0) big = 0;
    child_offsets(t, node, p, ch, e);
    l2l_node<DF>(node, p, nq, comp, ch, e, buf, &big, loc);
    if (DF && big) {
        __syncthreads();
        l2l_node<false>(node, p, nq, comp, ch, e, buf, &big, loc);
    }
}

// Shared memory of k_m2m / k_l2l: powers, components, dense expansions and
// the powers in the kernel's arithmetic.
size_t xlate_smem(int p, int ndense, int ncomp) {
    const int P1 = p + 1, nq = nT(p);
    return sizeof(double) * (2 * 8 * 3 * (size_t)P1 + (ncomp * nq + 1) / 2 + (size_t)ndense * P1 * P1 * P1);
}

// ---------------------------------------------------------------- L2P
// Block per leaf: the leaf's coefficients c = L_{t+u} h^|t+u| / u! (lengths
// in units of the leaf half-width h) staged from the table, then one work
// item per (particle, output t): nested Horner schemes over the output's
// coefficients.
constexpr int kL2pThreads = 128;

template <typename R>
__global__ void __launch_bounds__(kL2pThreads) k_l2p(const TreeDev t, const double* __restrict__ sx,
                                                     const double* __restrict__ sy, const double* __restrict__ sz,
                                                     int64_t n, int p, int f, const int* __restrict__ tab, L2pTab v,
                                                     const double* __restrict__ loc, double* __restrict__ fs) {
    extern __shared__ __align__(16) unsigned char sm_l2p_raw[];
    __shared__ double hp[kMaxP + 1];  // h^k
    __shared__ int seg[nT(3) + 1];  // field order <= 3
    R* coef = reinterpret_cast<R*>(sm_l2p_raw);
    const int nq = nT(p), nf = v.nf;
    const int leaf = t.leaves[blockIdx.x];
    const double h = t.r[leaf], ih = 1.0 / h;
    const double* L = loc + (size_t)leaf * nq;
    if (threadIdx.x <= p) {
        double w = 1.0;
        for (int k = 0; k < (int)threadIdx.x; ++k) w *= h;
        hp[threadIdx.x] = w;
    }
    if (threadIdx.x <= nf) seg[threadIdx.x] = tab[v.seg + threadIdx.x];
    __syncthreads();
    const int* wk = tab + v.wk;
    const double* fac = reinterpret_cast<const double*>(tab + v.fac);
    for (int e = threadIdx.x; e < v.ncoef; e += kL2pThreads) {
        const int w = wk[e];
        coef[e] = (R)(L[w & 0xffff] * hp[w >> 16] * fac[e]);
    }
    __syncthreads();
    const double cx = t.cx[leaf], cy = t.cy[leaf], cz = t.cz[leaf];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    for (int item = threadIdx.x; item < cnt * nf; item += kL2pThreads) {
        const int tq = item / cnt, k = s0 + item - tq * cnt;
        const R dx = (R)((sx[k] - cx) * ih), dy = (R)((sy[k] - cy) * ih), dz = (R)((sz[k] - cz) * ih);
        const int kt = order_of(tq), rem = p - kt;
        const R* c = coef + seg[tq];
        int b = 0;
        R hx = (R)0;
        for (int ux = rem; ux >= 0; --ux) {
            R hy = (R)0;
            for (int uy = rem - ux; uy >= 0; --uy) {
                R hz = (R)0;
                for (int uz = rem - ux - uy; uz >= 0; --uz) hz = hz * dz + c[b++];
                hy = hy * dy + hz;
            }
            hx = hx * dx + hy;
        }
        double s = 1.0;
        for (int a = 0; a < kt; ++a) s *= ih;  // kt <= 3
        fs[(size_t)tq * n + k] += (double)hx * s;
    }
}

int set_smem(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) FMM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return FMM_OK;
}

// P2M launch with KS = ceil(nq / NT) output slots per thread.
template <bool DF, int NM, int NT>
int launch_p2m(Workspace& ws, const Particles& P, const TreeDev& t, int p, const int* tab, const TabView& v,
               double* mom, cudaStream_t st) {
    const size_t sm = sizeof(double) * (size_t)p2m_stage_entries(p, NM) + sizeof(int) * (size_t)v.nq;
    const int ks = (v.nq + NT - 1) / NT;
#define FMM_P2M_CASE(KS)                                                                                          \
    case KS:                                                                                                      \
        FMM_TRY(set_smem((const void*)k_p2m<DF, NM, KS, NT>, sm));                                                \
        k_p2m<DF, NM, KS, NT><<<(unsigned)t.num_leaves, NT, sm, st>>>(t, ws.sx.as<double>(), ws.sy.as<double>(),  \
                                                                      ws.sz.as<double>(), ws.smc.as<double>(), P.n, \
                                                                      p, tab, v, mom);                            \
        break;
    switch (ks) {
        FMM_P2M_CASE(1)
        FMM_P2M_CASE(2)
        FMM_P2M_CASE(3)
        FMM_P2M_CASE(4)
        default:
            return FMM_EINVAL;
    }
#undef FMM_P2M_CASE
    return FMM_OK;
}

}  // namespace

int launch_p2m_m2m(Workspace& ws, const Particles& P, const TreeDev& t, int p, cudaStream_t st, bool df) {
    const int nq = nT(p);
    const int m = dim_to_order(P.dim);
    TabView v;
    FMM_TRY(ensure_tables(ws, p, &v, st));
    const int* tab = ws.xlate.as<int>();
    FMM_TRY(ws.mom.ensure(sizeof(double) * (size_t)t.num_nodes * nq));
    double* mom = ws.mom.as<double>();
    ws.wred_p = -1;  // new moments: the reduced weights are stale
    if (t.num_leaves > 0) {
        count_launches(1);
        const int nm = nT(m);
        if (df) {
            if (nm == 1) FMM_TRY((launch_p2m<true, 1, 128>(ws, P, t, p, tab, v, mom, st)));
            else if (nm == 4) FMM_TRY((launch_p2m<true, 4, 128>(ws, P, t, p, tab, v, mom, st)));
            else if (nm == 10) FMM_TRY((launch_p2m<true, 10, 128>(ws, P, t, p, tab, v, mom, st)));
            else return FMM_ENOTSUP;  // the double-float path takes multipole orders <= 2
        } else {
            if (nm == 1) FMM_TRY((launch_p2m<false, 1, 256>(ws, P, t, p, tab, v, mom, st)));
            else if (nm == 4) FMM_TRY((launch_p2m<false, 4, 256>(ws, P, t, p, tab, v, mom, st)));
            else if (nm == 10) FMM_TRY((launch_p2m<false, 10, 256>(ws, P, t, p, tab, v, mom, st)));
            else if (nm == 20) FMM_TRY((launch_p2m<false, 20, 256>(ws, P, t, p, tab, v, mom, st)));
            else return FMM_ENOTSUP;
        }
    }
    {
        const size_t sm = xlate_smem(p, 2, 4);
        FMM_TRY(set_smem((const void*)k_m2m<false>, sm));
        FMM_TRY(set_smem((const void*)k_m2m<true>, sm));
        for (int d = t.max_depth - 1; d >= 1; --d) {
            const int lo = t.level_start[d], hi = t.level_start[d + 1];
            if (hi <= lo) continue;
            count_launches(1);
            if (df)
                k_m2m<true><<<(unsigned)(hi - lo), kXThreads, sm, st>>>(t, t.level_nodes + lo, p, tab, v, mom);
            else
                k_m2m<false><<<(unsigned)(hi - lo), kXThreads, sm, st>>>(t, t.level_nodes + lo, p, tab, v, mom);
        }
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_l2l_l2p(Workspace& ws, const Particles& P, const TreeDev& t, int p, int field_order, bool fp32,
                   cudaStream_t st) {
    const int nq = nT(p);
    TabView v;
    FMM_TRY(ensure_tables(ws, p, &v, st));
    const int* tab = ws.xlate.as<int>();
    double* loc = ws.loc.as<double>();
    {
        const size_t sm = xlate_smem(p, 3, 1);
        FMM_TRY(set_smem((const void*)k_l2l<false>, sm));
        FMM_TRY(set_smem((const void*)k_l2l<true>, sm));
        for (int d = 1; d < t.max_depth; ++d) {
            const int lo = t.level_start[d], hi = t.level_start[d + 1];
            if (hi <= lo) continue;
            count_launches(1);
            if (fp32)
                k_l2l<true><<<(unsigned)(hi - lo), kXThreads, sm, st>>>(t, t.level_nodes + lo, p, tab, v, loc);
            else
                k_l2l<false><<<(unsigned)(hi - lo), kXThreads, sm, st>>>(t, t.level_nodes + lo, p, tab, v, loc);
        }
    }
    if (t.num_leaves > 0) {
        L2pTab lv;
        FMM_TRY(ensure_l2p_table(ws, p, field_order, &lv, st));
        const int* ltab = ws.l2pt.as<int>();
        count_launches(1);
        if (fp32) {
            const size_t sm = sizeof(float) * (size_t)lv.ncoef;
            FMM_TRY(set_smem((const void*)k_l2p<float>, sm));
            k_l2p<float><<<(unsigned)t.num_leaves, kL2pThreads, sm, st>>>(
                t, ws.sx.as<double>(), ws.sy.as<double>(), ws.sz.as<double>(), P.n, p, field_order, ltab, lv, loc,
                ws.fsorted.as<double>());
        } else {
            const size_t sm = sizeof(double) * (size_t)lv.ncoef;
            FMM_TRY(set_smem((const void*)k_l2p<double>, sm));
            k_l2p<double><<<(unsigned)t.num_leaves, kL2pThreads, sm, st>>>(
                t, ws.sx.as<double>(), ws.sy.as<double>(), ws.sz.as<double>(), P.n, p, field_order, ltab, lv, loc,
                ws.fsorted.as<double>());
        }
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

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
// The (output, term) index pairs of the convolutions are tabulated once per
// order on the host and staged in shared memory, so the inner loops are a
// table load and an FMA.  P2M runs a block per leaf over batches of
// particles (their scaled powers in shared memory); M2M and L2L a block per
// parent with all its children at once; L2P a thread per particle with the
// local expansion evaluated by nested Horner schemes in the leaf's length
// unit (FP32 in the mixed-precision path, where the local expansion's terms
// decrease with order and carry no cancellation between per-atom terms).
// P2M, M2M and L2L are FP64 in the plain path and double-float (FP32 pipe,
// exact products by FMA, ~48-bit sums) in the mixed path, M2M and L2L with
// an FP64 fallback for blocks whose powers or moments leave the range where
// FP32 exponents suffice.
#include <algorithm>
#include <vector>

#include "internal.h"

namespace fmm {

namespace {

__host__ __device__ constexpr int pack3(int x, int y, int z) { return x | (y << 8) | (z << 16); }
__device__ __forceinline__ int ux_(int c) { return c & 0xff; }
__device__ __forceinline__ int uy_(int c) { return (c >> 8) & 0xff; }
__device__ __forceinline__ int uz_(int c) { return (c >> 16) & 0xff; }

// Table layout (int32): comp[nq] | p2m_off[nq+1] | p2m[..] | m2m_off[nq+1] |
// m2m[..] | l2l_off[nq+1] | l2l[..]; entries pack two packed indices
// (low 16 bits, high 16 bits).
struct TabView {
    int nq, n_p2m, n_m2m, n_l2l;
    int comp, p2m_off, p2m, m2m_off, m2m, l2l_off, l2l, total;
};

TabView tab_view(int p, int n_p2m, int n_m2m, int n_l2l) {
    TabView v;
    v.nq = nT(p);
    v.n_p2m = n_p2m;
    v.n_m2m = n_m2m;
    v.n_l2l = n_l2l;
    int o = 0;
    v.comp = o;
    o += v.nq;
    v.p2m_off = o;
    o += v.nq + 1;
    v.p2m = o;
    o += n_p2m;
    v.m2m_off = o;
    o += v.nq + 1;
    v.m2m = o;
    o += n_m2m;
    v.l2l_off = o;
    o += v.nq + 1;
    v.l2l = o;
    o += n_l2l;
    v.total = o;
    return v;
}

int hidx(int x, int y, int z) { return nT(x + y + z - 1) + ((y + z) * (y + z + 1)) / 2 + z; }

// Builds (once per (p, m)) and uploads the index tables.
int ensure_tables(Workspace& ws, int p, int m, TabView* out, cudaStream_t st) {
    if (ws.xlate_p == p && ws.xlate_m == m) {
        *out = tab_view(p, ws.xlate_n[0], ws.xlate_n[1], ws.xlate_n[2]);
        return FMM_OK;
    }
    const int nq = nT(p), nm = nT(m);
    std::vector<int> comp(nq), xs(nq), ys(nq), zs(nq);
    for (int k = 0, q = 0; k <= p; ++k)
        for (int x = k; x >= 0; --x)
            for (int y = k - x; y >= 0; --y, ++q) {
                xs[q] = x;
                ys[q] = y;
                zs[q] = k - x - y;
                comp[q] = pack3(x, y, k - x - y);
            }
    std::vector<int> p2m_off(1, 0), p2m, m2m_off(1, 0), m2m, l2l_off(1, 0), l2l;
    for (int q = 0; q < nq; ++q) {
        for (int s = 0; s < std::min(nm, nq); ++s)
            if (xs[s] <= xs[q] && ys[s] <= ys[q] && zs[s] <= zs[q])
                p2m.push_back(s | (hidx(xs[q] - xs[s], ys[q] - ys[s], zs[q] - zs[s]) << 16));
        p2m_off.push_back((int)p2m.size());
        for (int u = 0; u < nq; ++u)
            if (xs[u] <= xs[q] && ys[u] <= ys[q] && zs[u] <= zs[q])
                m2m.push_back(u | (hidx(xs[q] - xs[u], ys[q] - ys[u], zs[q] - zs[u]) << 16));
        m2m_off.push_back((int)m2m.size());
        const int rem = p - (xs[q] + ys[q] + zs[q]);
        for (int u = 0; u < nT(rem); ++u) l2l.push_back(u | (hidx(xs[q] + xs[u], ys[q] + ys[u], zs[q] + zs[u]) << 16));
        l2l_off.push_back((int)l2l.size());
    }
    const TabView v = tab_view(p, (int)p2m.size(), (int)m2m.size(), (int)l2l.size());
    *out = v;
    std::vector<int> all((size_t)v.total);
    std::copy(comp.begin(), comp.end(), all.begin() + v.comp);
    std::copy(p2m_off.begin(), p2m_off.end(), all.begin() + v.p2m_off);
    std::copy(p2m.begin(), p2m.end(), all.begin() + v.p2m);
    std::copy(m2m_off.begin(), m2m_off.end(), all.begin() + v.m2m_off);
    std::copy(m2m.begin(), m2m.end(), all.begin() + v.m2m);
    std::copy(l2l_off.begin(), l2l_off.end(), all.begin() + v.l2l_off);
    std::copy(l2l.begin(), l2l.end(), all.begin() + v.l2l);
    FMM_TRY(ws.xlate.ensure(sizeof(int) * all.size()));
    FMM_CUDA_TRY(cudaMemcpyAsync(ws.xlate.p, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    ws.xlate_p = p;
    ws.xlate_m = m;
    ws.xlate_n[0] = v.n_p2m;
    ws.xlate_n[1] = v.n_m2m;
    ws.xlate_n[2] = v.n_l2l;
    return FMM_OK;
}

__device__ __forceinline__ void copy_ints(int* dst, const int* __restrict__ src, int n) {
    for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = src[e];
}

// 1/a and 1/a! for a = 0..2 kMaxP (no divisions on the FP64 pipe)
__constant__ double cInvInt[2 * kMaxP + 2] = {
#define FMM_X(a) ((a) == 0 ? 0.0 : 1.0 / (a)),
    FMM_X(0) FMM_X(1) FMM_X(2) FMM_X(3) FMM_X(4) FMM_X(5) FMM_X(6) FMM_X(7) FMM_X(8) FMM_X(9) FMM_X(10) FMM_X(11)
    FMM_X(12) FMM_X(13) FMM_X(14) FMM_X(15) FMM_X(16) FMM_X(17) FMM_X(18) FMM_X(19) FMM_X(20) FMM_X(21) FMM_X(22)
    FMM_X(23) FMM_X(24) FMM_X(25)
#undef FMM_X
};
__constant__ double cInvFact[kMaxP + 1] = {
#define FMM_F(a) (1.0 / cfact(a)),
    FMM_F(0) FMM_F(1) FMM_F(2) FMM_F(3) FMM_F(4) FMM_F(5) FMM_F(6) FMM_F(7) FMM_F(8) FMM_F(9) FMM_F(10) FMM_F(11)
    FMM_F(12)
#undef FMM_F
};
static_assert(kMaxP == 12, "inverse tables cover orders up to 12");

// e[a] = d^a / a!, a = 0..p
__device__ __forceinline__ void scaled_powers(double d, int p, double* e) {
    e[0] = 1.0;
    for (int a = 1; a <= p; ++a) e[a] = e[a - 1] * d * cInvInt[a];
}

// ---------------------------------------------------------------- P2M
constexpr int kP2mThreads = 128;
constexpr int kP2mBatch = 8;
constexpr int kMaxOut = (nT(kMaxP) + kP2mThreads - 1) / kP2mThreads;

// Product of two double-float pairs (hi, lo), renormalised.
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float s = p + e;
    return make_float2(s, e - (s - p));
}

// DF: accumulate in double-float pairs (FP32 arithmetic, exact products by
// FMA, ~48-bit sums) instead of FP64; used by the mixed-precision path, where
// the FP64 pipe is the bottleneck of this kernel.
template <bool DF>
__global__ void __launch_bounds__(kP2mThreads) k_p2m(const TreeDev t, const double* __restrict__ sx,
                                                     const double* __restrict__ sy, const double* __restrict__ sz,
                                                     const double* __restrict__ smc, int64_t n, int m, int p,
                                                     const int* __restrict__ tab, TabView v,
                                                     double* __restrict__ mom) {
    extern __shared__ __align__(16) double sm_p2m[];
    const int nq = v.nq, nm = nT(m), P1 = p + 1;
    double* dp = sm_p2m;                        // [kP2mBatch][nq]  (DF: float2 hi/lo)
    double* e = dp + kP2mBatch * nq;            // [kP2mBatch][3][p+1]
    double* ms = e + kP2mBatch * 3 * P1;        // [kP2mBatch][nm]  (DF: float2 hi/lo)
    int* comp = reinterpret_cast<int*>(ms + kP2mBatch * nm);
    int* off = comp + nq;
    int* terms = off + nq + 1;
    float2* dp2 = reinterpret_cast<float2*>(dp);
    float2* ms2 = reinterpret_cast<float2*>(ms);
    copy_ints(comp, tab + v.comp, nq);
    copy_ints(off, tab + v.p2m_off, nq + 1);
    copy_ints(terms, tab + v.p2m, v.n_p2m);
    const int leaf = t.leaves[blockIdx.x];
    const double cx = t.cx[leaf], cy = t.cy[leaf], cz = t.cz[leaf];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    double acc[kMaxOut];
    float ah[kMaxOut], al[kMaxOut];
#pragma unroll
    for (int r = 0; r < kMaxOut; ++r) {
        acc[r] = 0.0;
        ah[r] = al[r] = 0.0f;
    }
    __syncthreads();
    for (int b0 = 0; b0 < cnt; b0 += kP2mBatch) {
        const int nb = min(kP2mBatch, cnt - b0);
        if (threadIdx.x < 3 * nb) {
            const int b = threadIdx.x / 3, ax = threadIdx.x % 3, k = s0 + b0 + b;
            const double d = ax == 0 ? sx[k] - cx : (ax == 1 ? sy[k] - cy : sz[k] - cz);
            scaled_powers(d, p, e + (b * 3 + ax) * P1);
        }
        for (int idx = threadIdx.x; idx < nb * nm; idx += blockDim.x) {
            const int b = idx / nm, s = idx % nm;
            const double c = smc[(size_t)s * n + s0 + b0 + b];
            const double w = ((order_of(s) + 1) % 2) ? -c : c;  // back to M_s / s!
            if (DF) {
                const float hi = (float)w;
                ms2[b * nm + s] = make_float2(hi, (float)(w - (double)hi));
            } else {
                ms[b * nm + s] = w;
            }
        }
        __syncthreads();
        if (DF) {
            // scaled powers as double-float pairs, products on the FP32 pipe
            float2* e2 = reinterpret_cast<float2*>(e);
            __syncthreads();
            for (int idx = threadIdx.x; idx < nb * 3 * P1; idx += blockDim.x) {
                const double w = e[idx];
                const float hi = (float)w;
                e2[idx] = make_float2(hi, (float)(w - (double)hi));
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < nb * nq; idx += blockDim.x) {
                const int b = idx / nq, u = idx % nq;
                const int c = comp[u];
                const float2* eb = e2 + b * 3 * P1;
                dp2[b * nq + u] = df_mul(df_mul(eb[ux_(c)], eb[P1 + uy_(c)]), eb[2 * P1 + uz_(c)]);
            }
        } else {
            for (int idx = threadIdx.x; idx < nb * nq; idx += blockDim.x) {
                const int b = idx / nq, u = idx % nq;
                const int c = comp[u];
                const double* eb = e + b * 3 * P1;
                dp[b * nq + u] = eb[ux_(c)] * eb[P1 + uy_(c)] * eb[2 * P1 + uz_(c)];
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kMaxOut; ++r) {
            const int tq = threadIdx.x + kP2mThreads * r;
            if (tq < nq) {
                if (DF) {
                    float h = ah[r], l = al[r];
                    for (int j = off[tq]; j < off[tq + 1]; ++j) {
                        const int s = terms[j] & 0xffff, u = terms[j] >> 16;
                        for (int b = 0; b < nb; ++b) {
                            const float2 d = dp2[b * nq + u], w = ms2[b * nm + s];
                            const float pr = d.x * w.x;
                            float er = fmaf(d.x, w.x, -pr);
                            er = fmaf(d.x, w.y, er);
                            er = fmaf(d.y, w.x, er);
                            const float sum = h + pr;
                            const float bb = sum - h;
                            l += ((h - (sum - bb)) + (pr - bb)) + er;
                            h = sum;
                        }
                    }
                    ah[r] = h;
                    al[r] = l;
                } else {
                    double a = acc[r];
                    for (int j = off[tq]; j < off[tq + 1]; ++j) {
                        const int s = terms[j] & 0xffff, u = terms[j] >> 16;
                        for (int b = 0; b < nb; ++b) a = fma(dp[b * nq + u], ms[b * nm + s], a);
                    }
                    acc[r] = a;
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < kMaxOut; ++r) {
        const int tq = threadIdx.x + kP2mThreads * r;
        if (tq < nq) mom[(size_t)leaf * nq + tq] = DF ? (double)ah[r] + (double)al[r] : acc[r];
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
constexpr int kXThreads = 256;
constexpr int kXOut = (nT(kMaxP) + kXThreads - 1) / kXThreads;  // outputs per thread

// (hi, lo) FP32 pair of an FP64 value; *big set when it is outside the range
// where double-float products keep their precision.
__device__ __forceinline__ float2 to_df(double w, int* big) {
    if (fabs(w) > 1e30) *big = 1;
    const float hi = (float)w;
    return make_float2(hi, (float)(w - (double)hi));
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

// Arithmetic of the shifts: FP64, or double-float pairs on the FP32 pipe.
template <bool DF>
struct XOps;
template <>
struct XOps<false> {
    using V = double;
    struct Acc {
        double a = 0.0;
        __device__ __forceinline__ void mac(double x, double y) { a = fma(x, y, a); }
        __device__ __forceinline__ double val() const { return a; }
    };
    static __device__ __forceinline__ double in(double w, int*) { return w; }
    static __device__ __forceinline__ double out(double v) { return v; }
};
template <>
struct XOps<true> {
    using V = float2;
    struct Acc {
        float h = 0.0f, l = 0.0f;
        __device__ __forceinline__ void mac(float2 x, float2 y) { df_mac(x, y, h, l); }
        __device__ __forceinline__ float2 val() const {
            const float s = h + l;
            return make_float2(s, l - (s - h));
        }
    };
    static __device__ __forceinline__ float2 in(double w, int* big) { return to_df(w, big); }
    static __device__ __forceinline__ double out(float2 v) { return (double)v.x + (double)v.y; }
};

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
// as shifts along z (Y from X), y (X from Y) and x (into the accumulators of
// the thread's outputs).  Writes the result unless *big was raised.
template <bool DF>
__device__ __forceinline__ void m2m_node(const TreeDev& t, int node, int p, int nq, const int* comp, const int* ch,
                                         const double* e, void* buf, int* big, double* __restrict__ mom) {
    using O = XOps<DF>;
    using V = typename O::V;
    const int P1 = p + 1, n3 = P1 * P1 * P1;
    V* X = reinterpret_cast<V*>(buf);
    V* Y = X + n3;
    V* E = Y + n3;  // [8][3][p+1]
    const int nch = ch[8];
    for (int k = threadIdx.x; k < nch * 3 * P1; k += blockDim.x) E[k] = O::in(e[k], big);
    typename O::Acc acc[kXOut];
    for (int b = 0; b < nch; ++b) {
        const double* mc = mom + (size_t)ch[b] * nq;
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int cc = comp[q];
            X[d3(cc & 0xff, (cc >> 8) & 0xff, cc >> 16, P1)] = O::in(mc[q], big);
        }
        __syncthreads();
        const V* ex = E + b * 3 * P1;
        const V* ey = ex + P1;
        const V* ez = ey + P1;
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int cc = comp[q], x = cc & 0xff, y = (cc >> 8) & 0xff, z = cc >> 16;
            typename O::Acc s;
            for (int u = 0; u <= z; ++u) s.mac(ez[u], X[d3(x, y, z - u, P1)]);
            Y[d3(x, y, z, P1)] = s.val();
        }
        __syncthreads();
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int cc = comp[q], x = cc & 0xff, y = (cc >> 8) & 0xff, z = cc >> 16;
            typename O::Acc s;
            for (int u = 0; u <= y; ++u) s.mac(ey[u], Y[d3(x, y - u, z, P1)]);
            X[d3(x, y, z, P1)] = s.val();
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kXOut; ++r) {
            const int q = threadIdx.x + kXThreads * r;
            if (q < nq) {
                const int cc = comp[q], x = cc & 0xff, y = (cc >> 8) & 0xff, z = cc >> 16;
                for (int u = 0; u <= x; ++u) acc[r].mac(ex[u], X[d3(x - u, y, z, P1)]);
            }
        }
        __syncthreads();  // X is the next child's
    }
    if (DF && *big) return;
#pragma unroll
    for (int r = 0; r < kXOut; ++r) {
        const int q = threadIdx.x + kXThreads * r;
        if (q < nq) mom[(size_t)node * nq + q] = O::out(acc[r].val());
    }
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
    int* comp = reinterpret_cast<int*>(e + 8 * 3 * P1);          // [nq]
    void* buf = e + 8 * 3 * P1 + (nq + 1) / 2;                   // X, Y, E
    copy_ints(comp, tab + v.comp, nq);
    if (threadIdx.x == 0) big = 0;
    child_offsets(t, node, p, ch, e);
    m2m_node<DF>(t, node, p, nq, comp, ch, e, buf, &big, mom);
    if (DF) {
        __syncthreads();
        if (big) m2m_node<false>(t, node, p, nq, comp, ch, e, buf, &big, mom);
    }
}

// L2L of one parent into each child: L_t(child) += sum_u L_{t+u}(parent)
// d^u/u! (|t + u| <= p) as shifts along z (Y from X, the parent's
// expansion), y (Z from Y) and x (into the child's expansion).
template <bool DF>
__device__ __forceinline__ void l2l_node(int node, int p, int nq, const int* comp, const int* ch, const double* e,
                                         void* buf, int* big, double* __restrict__ loc) {
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
        double* lc = loc + (size_t)ch[b] * nq;
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int cc = comp[q], x = cc & 0xff, y = (cc >> 8) & 0xff, z = cc >> 16;
            typename O::Acc s;
            for (int u = 0; u <= p - x - y - z; ++u) s.mac(ex[u], Z[d3(x + u, y, z, P1)]);
            lc[q] += O::out(s.val());
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
size_t xlate_smem(int p, int ndense) {
    const int P1 = p + 1, nq = nT(p);
    return sizeof(double) * (2 * 8 * 3 * (size_t)P1 + (nq + 1) / 2 + (size_t)ndense * P1 * P1 * P1);
}

// ---------------------------------------------------------------- L2P
// Coefficients of output t (|t| <= f) in Horner order: ux, uy, uz descending,
// c = L_{t+u} h^|t+u| / u!  (lengths in units of the leaf half-width h).
template <typename R>
__global__ void __launch_bounds__(64) k_l2p(const TreeDev t, const double* __restrict__ sx,
                                            const double* __restrict__ sy, const double* __restrict__ sz, int64_t n,
                                            int p, int f, const double* __restrict__ loc, double* __restrict__ fs) {
    extern __shared__ __align__(16) unsigned char sm_l2p_raw[];
    __shared__ double hp[kMaxP + 1];  // h^k
    R* coef = reinterpret_cast<R*>(sm_l2p_raw);
    const int nq = nT(p), nf = nT(f);
    const int leaf = t.leaves[blockIdx.x];
    const double h = t.r[leaf], ih = 1.0 / h;
    const double* L = loc + (size_t)leaf * nq;
    if (threadIdx.x == 0) {
        double v = 1.0;
        for (int k = 0; k <= p; ++k) {
            hp[k] = v;
            v *= h;
        }
    }
    __syncthreads();
    // outputs tq of order k_t use nT(p - k_t) coefficients each, stored one
    // after the other
    int base = 0;
    for (int tq = 0; tq < nf; ++tq) {
        const int kt = order_of(tq);
        const int tx = comp_x(tq), ty = comp_y(tq), tz = comp_z(tq);
        const int rem = p - kt;
        const int cnt = nT(rem);
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            // e-th entry of the Horner order: decode (ux, uy, uz)
            int idx = e, ux = rem, uy = 0, uz = 0;
            for (ux = rem; ux >= 0; --ux) {
                const int blk = (rem - ux + 1) * (rem - ux + 2) / 2;
                if (idx < blk) break;
                idx -= blk;
            }
            for (uy = rem - ux; uy >= 0; --uy) {
                const int blk = rem - ux - uy + 1;
                if (idx < blk) break;
                idx -= blk;
            }
            uz = rem - ux - uy - idx;
            const int w = pidx(tx + ux, ty + uy, tz + uz);
            const double s = hp[kt + ux + uy + uz] * (cInvFact[ux] * cInvFact[uy] * cInvFact[uz]);
            coef[base + e] = (R)(L[w] * s);
        }
        base += cnt;
    }
    __syncthreads();
    const double cx = t.cx[leaf], cy = t.cy[leaf], cz = t.cz[leaf];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    for (int k = s0 + threadIdx.x; k < s0 + cnt; k += blockDim.x) {
        const R dx = (R)((sx[k] - cx) * ih), dy = (R)((sy[k] - cy) * ih), dz = (R)((sz[k] - cz) * ih);
        int b = 0;
        for (int tq = 0; tq < nf; ++tq) {
            const int kt = order_of(tq);
            const int rem = p - kt;
            R hx = (R)0;
            for (int ux = rem; ux >= 0; --ux) {
                R hy = (R)0;
                for (int uy = rem - ux; uy >= 0; --uy) {
                    R hz = (R)0;
                    for (int uz = rem - ux - uy; uz >= 0; --uz) hz = hz * dz + coef[b++];
                    hy = hy * dy + hz;
                }
                hx = hx * dx + hy;
            }
            double s = 1.0;
            for (int a = 0; a < kt; ++a) s *= ih;  // kt <= 2
            fs[(size_t)tq * n + k] += (double)hx * s;
        }
    }
}

size_t l2p_coef_count(int p, int f) {
    size_t c = 0;
    for (int tq = 0; tq < nT(f); ++tq) c += nT(p - order_of(tq));
    return c;
}

int set_smem(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) FMM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return FMM_OK;
}

}  // namespace

int launch_p2m_m2m(Workspace& ws, const Particles& P, const TreeDev& t, int p, cudaStream_t st, bool df) {
    const int nq = nT(p);
    const int m = dim_to_order(P.dim);
    TabView v;
    FMM_TRY(ensure_tables(ws, p, m, &v, st));
    const int* tab = ws.xlate.as<int>();
    FMM_TRY(ws.mom.ensure(sizeof(double) * (size_t)t.num_nodes * nq));
    double* mom = ws.mom.as<double>();
    {
        const int nm = nT(m);
        const size_t sm = sizeof(double) * (kP2mBatch * (size_t)nq + kP2mBatch * 3 * (p + 1) + kP2mBatch * nm) +
                          sizeof(int) * (2 * (size_t)nq + 1 + v.n_p2m);
        FMM_TRY(set_smem((const void*)k_p2m<false>, sm));
        FMM_TRY(set_smem((const void*)k_p2m<true>, sm));
        if (t.num_leaves > 0) {
            count_launches(1);
            if (df)
                k_p2m<true><<<(unsigned)t.num_leaves, kP2mThreads, sm, st>>>(
                    t, ws.sx.as<double>(), ws.sy.as<double>(), ws.sz.as<double>(), ws.smc.as<double>(), P.n, m, p,
                    tab, v, mom);
            else
                k_p2m<false><<<(unsigned)t.num_leaves, kP2mThreads, sm, st>>>(
                    t, ws.sx.as<double>(), ws.sy.as<double>(), ws.sz.as<double>(), ws.smc.as<double>(), P.n, m, p,
                    tab, v, mom);
        }
    }
    {
        const size_t sm = xlate_smem(p, 2);
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
    FMM_TRY(ensure_tables(ws, p, dim_to_order(P.dim), &v, st));
    const int* tab = ws.xlate.as<int>();
    double* loc = ws.loc.as<double>();
    {
        const size_t sm = xlate_smem(p, 3);
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
        const size_t ncoef = l2p_coef_count(p, field_order);
        count_launches(1);
        if (fp32) {
            const size_t sm = sizeof(float) * ncoef;
            FMM_TRY(set_smem((const void*)k_l2p<float>, sm));
            k_l2p<float><<<(unsigned)t.num_leaves, 64, sm, st>>>(t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                                 ws.sz.as<double>(), P.n, p, field_order, loc,
                                                                 ws.fsorted.as<double>());
        } else {
            const size_t sm = sizeof(double) * ncoef;
            FMM_TRY(set_smem((const void*)k_l2p<double>, sm));
            k_l2p<double><<<(unsigned)t.num_leaves, 64, sm, st>>>(t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                                  ws.sz.as<double>(), P.n, p, field_order, loc,
                                                                  ws.fsorted.as<double>());
        }
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

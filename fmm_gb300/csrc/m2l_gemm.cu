// M2L as dense matrix products grouped by displacement (exact-coefficient
// modes; the reference's per-pair M2L is src/fmm.F90:826-882).
//
// Octree cells are cubes on a grid: the centre displacement of two cells is an
// integer multiple D of the smaller cell's half-width, and a pair's
// reduced-basis M2L operator depends only on D, the level difference and the
// pair's expansion order q.  The far pairs are sorted by that key; each group
// shares one operator G ((q+1)^2 x (q+1)^2, from the restricted tensor T of
// the group's displacement, computed once per group in FP64), and the group's
// pairs are the columns of one product C = G W.  FP32 products run on the
// tensor cores (tcgen05, kind::tf32 with operands split into two TF32 parts,
// three products per term, FP32 accumulators in tensor memory); FP64
// products, and FP32 ones on request, on the CUDA cores as register-tiled
// blocks.  Per-pair columns go to a buffer in target-sorted order and are
// summed per target with compensated sums.
//
// Units: per-node weights w'_s = w^_s / h_j^|s|, per-target locals
// L'_f = h_i^(|f|+1) L_f, tensor T(D_c) at the displacement in units of the
// coarser cell's half-width h_c; then G_fs = a^(|f|+1) b^|s| T_{s+f}(D_c)
// with a = h_i/h_c, b = h_j/h_c (powers of two, at most 1), so all operands
// are O(1) and the FP32 products stay in range.
#include <algorithm>

#include <cub/cub.cuh>

#include <cstdlib>
#include <cstring>

#include "internal.h"
#include "m2l_basis.cuh"
#include "umma.cuh"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

constexpr int kFallback = 63;            // key code of pairs without a grid displacement
// Key layout (46 bits, so the radix sort needs 6 digit passes): level
// difference + 31 (6 bits) | order (4) | Dx, Dy, Dz + kDOff (12 bits each).
constexpr int kKeyBits = 46;
constexpr int64_t kDOff = 1 << 11;       // offset of the 12-bit displacement fields
constexpr int kTaskCols = 512;           // pairs (columns) per product block
constexpr int kGemmThreads = 128;        // 16 row groups x 8 column groups
constexpr int kTcRows = 128;             // tensor-core MMA M: operator rows f per half
constexpr int kTcPairs = 256;            // tensor-core MMA N: pairs per task

// Operator halves of 128 rows f for order q (two above order 10).
__host__ __device__ __forceinline__ int tc_halves(int q) { return (q + 1) * (q + 1) > kTcRows ? 2 : 1; }

__global__ void k_far_targets(int M, const int32_t* __restrict__ off, int32_t* __restrict__ tgt) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= M) return;
    for (int q = off[i] + lane; q < off[i + 1]; q += 32) tgt[q] = i;
}

// w'_s = w^_s / h^|s| per node (h the node's half-width).
// (rows of ld >= nr entries, zero padded)
template <typename R>
__global__ void k_scale_weights(int M, int nr, int ld, const double* __restrict__ wred, const double* __restrict__ h,
                                R* __restrict__ wsc) {
    // warp per node: lane j holds ih^j (the same sequential product for every
    // component of order j), components across the lanes
    const int node = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (node >= M) return;
    const double ih = 1.0 / h[node];
    double pw = 1.0;
    for (int u = 0; u < min(lane, 2 * kMaxP); ++u) pw *= ih;
    for (int s0 = 0; s0 < ld; s0 += 32) {
        const int s = s0 + lane;
        int k = 0;
        while ((k + 1) * (k + 1) <= s) ++k;  // order of reduced component s
        const double sc = __shfl_sync(0xffffffffu, pw, min(k, 31));
        if (s < ld) wsc[(size_t)node * ld + s] = s < nr ? (R)(wred[(size_t)node * nr + s] * sc) : (R)0;
    }
}

// Group key of every far pair: level difference, expansion order and integer
// displacement in units of the smaller half-width; pairs off the grid (or
// with out-of-range fields) get unique keys of their own (code 63 | index).
// With FP32 node data (chi: centre hi parts; clo: low parts, half-width in
// w) the displacement is formed from the double-float centres on the FP32
// pipe; its error (a few 1e-8 relative of the displacement, up to ~1e-4 cell
// units at the largest encodable displacement) stays far below the 1e-3
// tolerance of the integer test.  Without them, FP64 with a 1e-6 tolerance.
__global__ void k_m2l_keys(int64_t nfar, const TreeDev t, const int32_t* __restrict__ tgt, int p, int oclass,
                           const float4* __restrict__ chi, const float4* __restrict__ clo,
                           uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nfar) return;
    const int i = tgt[q], j = t.far_src[q];
    const int ord = t.far_ord ? min((int)t.far_ord[q], p) : p;
    // half-widths are the root's divided by powers of two: 1/h times an
    // integer multiple of h stays within rounding of that integer
    float rx, ry, rz, ex, ey, ez, tol;
    if (chi) {
        const float4 ci = chi[i], cj = chi[j], li = clo[i], lj = clo[j];
        const float ihf = 1.0f / fminf(li.w, lj.w);
        const float dx = ((ci.x - cj.x) + (li.x - lj.x)) * ihf, dy = ((ci.y - cj.y) + (li.y - lj.y)) * ihf,
                    dz = ((ci.z - cj.z) + (li.z - lj.z)) * ihf;
        rx = rintf(dx);
        ry = rintf(dy);
        rz = rintf(dz);
        ex = fabsf(dx - rx);
        ey = fabsf(dy - ry);
        ez = fabsf(dz - rz);
        tol = 1e-3f;
    } else {
        const double ihf = 1.0 / fmin(t.r[i], t.r[j]);
        const double dx = (t.cx[i] - t.cx[j]) * ihf, dy = (t.cy[i] - t.cy[j]) * ihf, dz = (t.cz[i] - t.cz[j]) * ihf;
        const double Rx = rint(dx), Ry = rint(dy), Rz = rint(dz);
        rx = (float)Rx;
        ry = (float)Ry;
        rz = (float)Rz;
        ex = (float)fabs(dx - Rx);
        ey = (float)fabs(dy - Ry);
        ez = (float)fabs(dz - Rz);
        tol = 1e-6f;
    }
    const int dl = t.depth[i] - t.depth[j];
    const int oc = (ord + oclass - 1) / oclass;  // order class: the group takes its pairs' highest order
    const float lim = (float)(kDOff - 1);
    const bool grid = ex < tol && ey < tol && ez < tol && fabsf(rx) <= lim && fabsf(ry) <= lim && fabsf(rz) <= lim &&
                      dl > -31 && dl < 31;
    uint64_t key;
    if (grid)
        key = ((uint64_t)(dl + 31) << 40) | ((uint64_t)oc << 36) | ((uint64_t)((int64_t)rx + kDOff) << 24) |
              ((uint64_t)((int64_t)ry + kDOff) << 12) | (uint64_t)((int64_t)rz + kDOff);
    else
        key = ((uint64_t)kFallback << 40) | (uint64_t)q;
    keys[q] = key;
    vals[q] = (int32_t)q;
}

// One warp per group: restricted tensor T(D_c) of orders <= 2q in FP64 by the
// Hermite recursion (two level buffers in shared memory), stored as R, with
// the group's order and unit ratios a, b.
template <typename R>
__global__ void __launch_bounds__(128) k_group_tensor(int ngroups, const uint64_t* __restrict__ ukeys,
                                                      const int32_t* __restrict__ gstart,
                                                      const int32_t* __restrict__ svals,
                                                      const int32_t* __restrict__ tgt, const TreeDev t, int p,
                                                      int ldT, R* __restrict__ gT, int32_t* __restrict__ gq,
                                                      float2* __restrict__ gab) {
    extern __shared__ double smg[];
    const int N = 2 * p, nTr = rbase(N + 1);
    int2* rule = reinterpret_cast<int2*>(smg);
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* TA = smg + nTr + wib * (2 * nTr + N + 1);
    double* TB = TA + nTr;
    double* gsh = TB + nTr;
    for (int e = threadIdx.x; e < nTr; e += blockDim.x) rule[e] = restricted_rule(e);
    __syncthreads();
    const int g = blockIdx.x * (blockDim.x >> 5) + wib;
    if (g >= ngroups) return;
    const uint64_t key = ukeys[g];
    const int pos0 = svals[gstart[g]];
    const int i = tgt[pos0], j = t.far_src[pos0];
    // the group's order: the highest of its pairs' orders
    int q = 0;
    for (int k = gstart[g] + lane; k < gstart[g + 1]; k += 32)
        q = max(q, t.far_ord ? min((int)t.far_ord[svals[k]], p) : p);
    for (int off = 16; off > 0; off >>= 1) q = max(q, __shfl_xor_sync(0xffffffffu, q, off));
    const double hi = t.r[i], hj = t.r[j], hc = fmax(hi, hj);
    const double X = (t.cx[i] - t.cx[j]) / hc, Y = (t.cy[i] - t.cy[j]) / hc, Z = (t.cz[i] - t.cz[j]) / hc;
    const int Nq = 2 * q;
    const double r2 = X * X + Y * Y + Z * Z;
    const double rinv = 1.0 / sqrt(r2), rinv2 = rinv * rinv;
    if (lane <= Nq) {
        double v = rinv, c = 1.0;
        for (int jj = 1; jj <= lane; ++jj) {
            v *= rinv2;
            c *= -(double)(2 * jj - 1);
        }
        gsh[lane] = c * v;
    }
    __syncwarp();
    double* A = TA;
    double* B = TB;
    if (lane == 0) A[0] = gsh[Nq];
    __syncwarp();
    for (int lev = Nq - 1; lev >= 0; --lev) {
        const int lim = rbase(Nq - lev + 1);
        for (int e = lane; e < lim; e += 32) {
            double v;
            if (e == 0) {
                v = gsh[lev];
            } else {
                const int2 ru = rule[e];
                const int dir = ru.x >> 16, cnt = ru.y >> 16;
                const double crd = dir == 0 ? X : (dir == 1 ? Y : Z);
                v = crd * A[ru.x & 0xffff];
                if (cnt > 0) v += (double)cnt * A[ru.y & 0xffff];
            }
            B[e] = v;
        }
        __syncwarp();
        double* tmp = A;
        A = B;
        B = tmp;
    }
    R* out = gT + (size_t)g * ldT;
    for (int e = lane; e < rbase(Nq + 1); e += 32) out[e] = (R)A[e];
    if (lane == 0) {
        gq[g] = q;
        gab[g] = make_float2((float)(hi / hc), (float)(hj / hc));
    }
}

// Tasks of up to `cols` pairs of one group: counts, then (group, first
// column).  cols < 0: tensor-core tasks of kTcPairs pairs and one operator
// half each, (group, 2 x first column + half).
__global__ void k_task_counts(int ng, int cols, const int32_t* __restrict__ gq, const int32_t* __restrict__ gstart,
                              int32_t* __restrict__ tcnt) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > ng) return;
    if (g == ng) {
        tcnt[g] = 0;
        return;
    }
    const int n = gstart[g + 1] - gstart[g];
    tcnt[g] = cols > 0 ? (n + cols - 1) / cols : (n + kTcPairs - 1) / kTcPairs * tc_halves(gq[g]);
}

__global__ void k_fill_tasks(int ng, int cols, const int32_t* __restrict__ gq, const int32_t* __restrict__ gstart,
                             const int32_t* __restrict__ toff, int2* __restrict__ tasks) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int n = toff[g + 1] - toff[g];
    if (cols > 0) {
        for (int k = 0; k < n; ++k) tasks[toff[g] + k] = make_int2(g, k * cols);
    } else {
        const int h = tc_halves(gq[g]);
        for (int k = 0; k < n; ++k) tasks[toff[g] + k] = make_int2(g, 2 * kTcPairs * (k / h) + k % h);
    }
}

// Shared-memory plan of the product kernel (elements of R unless noted).
template <typename R, int CPT>
struct GemmSmem {
    static constexpr int TN = 8 * CPT;                // columns per tile
    static constexpr int VS = 16 / (int)sizeof(R);    // weights per 16-byte load
    int nrmax, rmmax, nTr;
    size_t off_dec, off_pow, off_T, off_col, off_G, bytes;
    __host__ __device__ GemmSmem(int p) {
        nrmax = (p + 1) * (p + 1);
        rmmax = 16 * ((nrmax + 15) / 16);
        nTr = rbase(2 * p + 1);
        size_t o = 0;
        off_dec = o;
        o += sizeof(int) * nrmax;
        o = (o + 15) & ~(size_t)15;
        off_pow = o;
        o += sizeof(R) * 32;
        off_T = o;
        o += sizeof(R) * nTr;
        o = (o + 15) & ~(size_t)15;
        off_col = o;  // the task's pair positions and source nodes
        o += sizeof(int) * 2 * kTaskCols;
        off_G = o;
        o += sizeof(R) * (size_t)((nrmax + VS - 1) / VS * VS) * rmmax;
        bytes = o;
    }
};

// Row stride of the per-node weights: (p+1)^2 rounded up to 16 bytes.
template <typename R>
__host__ __device__ constexpr int wsc_ld(int nr) {
    return (nr + 16 / (int)sizeof(R) - 1) / (16 / (int)sizeof(R)) * (16 / (int)sizeof(R));
}

template <typename R>
struct Vec;
template <>
struct Vec<float> {
    using T = float4;
    __device__ static __forceinline__ void get(const T& v, float* o) {
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
};
template <>
struct Vec<double> {
    using T = double2;
    __device__ static __forceinline__ void get(const T& v, double* o) {
        o[0] = v.x; o[1] = v.y;
    }
};

// RT consecutive operator rows as 16-byte loads where the alignment allows
// (row blocks of RT elements start at multiples of RT).
template <typename R, int RT>
__device__ __forceinline__ void load_rows(const R* p, R (&v)[RT]) {
    constexpr int VS = 16 / (int)sizeof(R);
    if constexpr (RT % VS == 0) {
        using V = typename Vec<R>::T;
#pragma unroll
        for (int k = 0; k < RT / VS; ++k) Vec<R>::get(reinterpret_cast<const V*>(p)[k], v + VS * k);
    } else if constexpr (sizeof(R) == 4 && RT % 2 == 0) {
#pragma unroll
        for (int k = 0; k < RT / 2; ++k) {
            const float2 x = reinterpret_cast<const float2*>(p)[k];
            v[2 * k] = x.x;
            v[2 * k + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < RT; ++k) v[k] = p[k];
    }
}

// Columns [c_begin, c_begin + kTaskCols) of one group: C = G W for tiles of
// TN pairs; thread (rg, cg) owns rows rg*RT + k (k < RT) and columns
// cg*CPT .. cg*CPT + CPT - 1 of each tile.  G^T sits in shared memory
// (s-major); each thread streams its columns' weights straight from global
// memory (L1/L2-resident), VS consecutive s per 16-byte load, so the tile loop
// needs no block barrier.
template <typename R, int RT, int CPT>
__device__ __forceinline__ void gemm_task(const GemmSmem<R, CPT>& L, char* sm, int c_begin, int tcols, int nrq,
                                          int cnt, int gs,
                                          const int32_t* __restrict__ svals, const int32_t* __restrict__ far_src,
                                          const R* __restrict__ wsc, int ldw, R* __restrict__ gout, int ldo) {
    constexpr int TN = GemmSmem<R, CPT>::TN;
    constexpr int VS = GemmSmem<R, CPT>::VS;
    constexpr int RM = 16 * RT;
    using V = typename Vec<R>::T;
    const int tid = threadIdx.x;
    const int rg = tid & 15, cg = tid >> 4;
    const int* dec = reinterpret_cast<const int*>(sm + L.off_dec);
    const R* apow = reinterpret_cast<const R*>(sm + L.off_pow);
    const R* bpow = apow + 16;
    const R* Tsh = reinterpret_cast<const R*>(sm + L.off_T);
    R* G = reinterpret_cast<R*>(sm + L.off_G);
    int* cpos = reinterpret_cast<int*>(sm + L.off_col);
    int* csrc = cpos + kTaskCols;
    const int nrv = (nrq + VS - 1) / VS * VS;
    const int c_end = min(cnt, c_begin + tcols);
    // the task's columns: pair positions and source nodes (loaded once)
    for (int i = tid; i < c_end - c_begin; i += kGemmThreads) {
        const int pos = svals[gs + c_begin + i];
        cpos[i] = pos;
        csrc[i] = far_src[pos];
    }
    // operator G^T (s-major, RM rows per s; rows f >= nrq and s >= nrq zero)
    for (int e = tid; e < nrv * RM; e += kGemmThreads) {
        const int s = e / RM, f = e - s * RM;
        R v = (R)0;
        if (f < nrq && s < nrq) {
            const int cs = dec[s], cf = dec[f];
            const int x = (cs & 0xff) + (cf & 0xff), y = ((cs >> 8) & 0xff) + ((cf >> 8) & 0xff),
                      z = ((cs >> 16) & 0xff) + ((cf >> 16) & 0xff);
            v = apow[(cf >> 24) + 1] * bpow[cs >> 24] * Tsh[ridx(x, y, z)];
        }
        G[e] = v;
    }
    __syncthreads();
    for (int cb = c_begin; cb < c_end; cb += TN) {
        int pos[CPT];
        const V* wp[CPT];
#pragma unroll
        for (int l = 0; l < CPT; ++l) {
            const int c = cb + cg * CPT + l;
            pos[l] = c < c_end ? c : -1;  // result row: the pair's place in its group
            wp[l] = pos[l] >= 0 ? reinterpret_cast<const V*>(wsc + (size_t)csrc[c - c_begin] * ldw) : nullptr;
        }
        R acc[RT][CPT];
#pragma unroll
        for (int k = 0; k < RT; ++k)
#pragma unroll
            for (int l = 0; l < CPT; ++l) acc[k][l] = (R)0;
        const R* Gp = G + rg * RT;  // this thread's RT consecutive rows
        for (int s0 = 0; s0 < nrv; s0 += VS) {
            R wv[CPT][VS];
#pragma unroll
            for (int l = 0; l < CPT; ++l) {
                if (wp[l]) {
                    Vec<R>::get(wp[l][s0 / VS], wv[l]);
                } else {
#pragma unroll
                    for (int u = 0; u < VS; ++u) wv[l][u] = (R)0;
                }
            }
#pragma unroll
            for (int u = 0; u < VS; ++u) {
                R gv[RT];
                load_rows<R, RT>(Gp + (s0 + u) * RM, gv);
#pragma unroll
                for (int k = 0; k < RT; ++k)
#pragma unroll
                    for (int l = 0; l < CPT; ++l) acc[k][l] = fma(gv[k], wv[l][u], acc[k][l]);
            }
        }
        // the group's rows are ldo = (q+1)^2 rounded up to kRowUnit entries
        // each (zeros above the pair's order)
#pragma unroll
        for (int l = 0; l < CPT; ++l) {
            if (pos[l] >= 0) {
                R* o = gout + (size_t)pos[l] * ldo;
#pragma unroll
                for (int k = 0; k < RT; ++k) {
                    const int f = rg * RT + k;
                    if (f < nrq)
                        o[f] = acc[k][l];
                    else if (f < ldo)
                        o[f] = (R)0;
                }
                for (int f = RM + rg; f < ldo; f += 16) o[f] = (R)0;
            }
        }
    }
}

// Result rows: group g's rows start at rowbase[g] x kRowUnit entries, one
// row of (q+1)^2 rounded up to kRowUnit entries (32 bytes in FP32, one DRAM
// sector) per pair in group order.
constexpr int kRowUnit = 8;
__host__ __device__ __forceinline__ int row_len(int q) {
    return ((q + 1) * (q + 1) + kRowUnit - 1) / kRowUnit * kRowUnit;
}

// tcols: pairs per task (at most kTaskCols); tasks of order < qmin are left
// to the tensor-core kernel.
template <typename R, int CPT>
__global__ void __launch_bounds__(kGemmThreads) k_m2l_gemm(const int2* __restrict__ tasks, int tcols, int qmin,
                                                           int p,
                                                           const int32_t* __restrict__ gstart,
                                                           const int32_t* __restrict__ gq,
                                                           const float2* __restrict__ gab, const R* __restrict__ gT,
                                                           int ldT, const int32_t* __restrict__ svals,
                                                           const int32_t* __restrict__ far_src,
                                                           const R* __restrict__ wsc, R* __restrict__ out,
                                                           const int32_t* __restrict__ rowbase) {
    extern __shared__ __align__(16) char sm_gemm[];
    const GemmSmem<R, CPT> L(p);
    const int nr = (p + 1) * (p + 1);
    const int2 task = tasks[blockIdx.x];
    const int g = task.x;
    const int q = gq[g], nrq = (q + 1) * (q + 1);
    if (q < qmin) return;
    const int gs = gstart[g], cnt = gstart[g + 1] - gs;
    int* dec = reinterpret_cast<int*>(sm_gemm + L.off_dec);
    R* apow = reinterpret_cast<R*>(sm_gemm + L.off_pow);
    R* bpow = apow + 16;
    R* Tsh = reinterpret_cast<R*>(sm_gemm + L.off_T);
    for (int e = threadIdx.x; e < nrq; e += kGemmThreads) dec[e] = qcomp(e);
    if (threadIdx.x < 16) {
        const float2 ab = gab[g];
        R a = (R)1, b = (R)1;
        for (int u = 0; u < (int)threadIdx.x; ++u) {
            a *= (R)ab.x;
            b *= (R)ab.y;
        }
        apow[threadIdx.x] = a;
        bpow[threadIdx.x] = b;
    }
    const int nTq = rbase(2 * q + 1);
    for (int e = threadIdx.x; e < nTq; e += kGemmThreads) Tsh[e] = gT[(size_t)g * ldT + e];
    __syncthreads();
    const int rt = (nrq + 15) / 16;
    switch (rt) {
#define FMM_GEMM_CASE(K)                                                                                     \
    case K:                                                                                                  \
        gemm_task<R, K, CPT>(L, sm_gemm, task.y, tcols, nrq, cnt, gs, svals, far_src, wsc, wsc_ld<R>(nr),     \
                             out + (size_t)rowbase[g] * kRowUnit, row_len(q));                                      \
        break;
        FMM_GEMM_CASE(1)
        FMM_GEMM_CASE(2)
        FMM_GEMM_CASE(3)
        FMM_GEMM_CASE(4)
        FMM_GEMM_CASE(5)
        FMM_GEMM_CASE(6)
        FMM_GEMM_CASE(7)
        FMM_GEMM_CASE(8)
        FMM_GEMM_CASE(9)
        FMM_GEMM_CASE(10)
        FMM_GEMM_CASE(11)
#undef FMM_GEMM_CASE
        default:
            break;
    }
}

// ---------------------------------------------------------------------------
// Tensor-core product.  A task is up to 256 pairs of one group and one half
// of its operator: D = G W^T with G the operator half (f x s, M = 128 rows
// f), W the pairs' weights (pairs x s, N = 256) and K = (q+1)^2
// in chunks of 8 (one MMA K step).  Both operands are split into TF32 parts,
// x = hi + lo, and D accumulates G_hi W_hi + G_hi W_lo + G_lo W_hi in FP32
// (the dropped G_lo W_lo and the rounding of the parts leave about 2^-22 of
// each term).  The parts are prepared once in global memory in the operand
// layout: per node the weights, per group the operator, chunk by chunk.
// Warp roles in a persistent block (one per SM):
//   warps 0-1  producers: per chunk, one bulk (TMA) copy of the operator
//              chunk and 16-byte cp.async gathers of the 256 pairs' weights
//              into a ring of shared-memory stages, completing on the
//              stage's full mbarrier; a stage is refilled once the MMAs that
//              read it have committed to its empty mbarrier;
//   warp 2     one thread issues the MMAs into one of two tensor-memory
//              accumulators (256 columns each) and commits the finished task;
//   warps 3+   epilogue (four per tensor-memory sub-partition, each a
//              quarter of the columns): each reads its 32 lanes (rows f),
//              32 columns (pairs) per wait, and writes, per pair, 32
//              consecutive entries of the pair's result row (one aligned
//              128-byte line), then frees the accumulator.
// The two accumulators let the epilogue of one task overlap the MMAs of the
// next.  Orders above 10 ((q+1)^2 > 128 rows f) have two operator halves,
// each a task of its own over the same pairs.
constexpr int kTcKC = 8;           // reduced components per chunk (one MMA K step)
constexpr int kTcStages = 8;
constexpr int kTcProducers = 64;   // warps 0-1
constexpr int kTcMmaWarp = 2;
constexpr int kTcEpiWarps = 16;    // warps 3 .. 2 + kTcEpiWarps
constexpr int kTcThreads = 32 * (3 + kTcEpiWarps);
constexpr int kTcEpiBatch = 2;     // tensor-memory loads (16 columns each) per wait
constexpr uint32_t kTcCols = 512;  // two accumulators of kTcPairs columns
constexpr long long kTcWaitCycles = 4000000000LL;  // about 2 s at 2 GHz

// Float offset of element (r, k) in a K-major, unswizzled chunk kTcKC wide:
// core matrices of 8 rows x 4 elements (128 bytes), K-adjacent ones 128 bytes
// apart (LBO), row groups kTcKC / 4 * 128 bytes apart (SBO).
__host__ __device__ constexpr int tc_off(int r, int k) {
    return (r >> 3) * (kTcKC * 8) + (k >> 2) * 32 + (r & 7) * 4 + (k & 3);
}
static_assert(tc_off(9, 6) == 64 + 32 + 4 + 2, "operand layout: row groups of 8, K groups of 4");

struct TcSmem {
    static constexpr int g_floats = kTcRows * kTcKC;   // one TF32 part of an operator chunk
    static constexpr int w_floats = kTcPairs * kTcKC;  // one TF32 part of a weight chunk
    static constexpr size_t stage_bytes = sizeof(float) * 2 * (g_floats + w_floats);
    static constexpr size_t off_bar = kTcStages * stage_bytes;
    // full[S], empty[S], acc_full[2], acc_empty[2]
    static constexpr size_t off_tmem = off_bar + sizeof(uint64_t) * (2 * kTcStages + 4);
    static constexpr size_t bytes = off_tmem + 16;
};

// Per-node weights as TF32 parts, chunk by chunk: [chunk][hi KC | lo KC].
__global__ void k_split_weights(int64_t total, int nr, int ldw, int ldk, const float* __restrict__ wsc,
                                float* __restrict__ wsp) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = e / ldk;
        const int s = (int)(e - node * ldk);
        const float v = s < nr ? wsc[node * ldw + s] : 0.0f;
        float h, l;
        umma::split_tf32(v, h, l);
        float* o = wsp + node * 2 * ldk + (s / kTcKC) * 2 * kTcKC + (s % kTcKC);
        o[0] = h;
        o[kTcKC] = l;
    }
}

// Rows of each group in units of kRowUnit entries (scanned into rowbase).
__global__ void k_row_sizes(int ng, const int32_t* __restrict__ gstart, const int32_t* __restrict__ gq,
                            int32_t* __restrict__ rsz) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > ng) return;
    rsz[g] = g < ng ? (gstart[g + 1] - gstart[g]) * (row_len(gq[g]) / kRowUnit) : 0;
}

// Row of every far pair, indexed in target order (svals maps group order to
// target order), in units of kRowUnit entries.  Warp per group.
__global__ void k_row_offsets(int ng, const int32_t* __restrict__ gstart, const int32_t* __restrict__ gq,
                              const int32_t* __restrict__ rowbase, const int32_t* __restrict__ svals,
                              int32_t* __restrict__ roff) {
    const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (g >= ng) return;
    const int lane = threadIdx.x & 31, u = row_len(gq[g]) / kRowUnit;
    for (int k = gstart[g] + lane; k < gstart[g + 1]; k += 32) roff[svals[k]] = rowbase[g] + (k - gstart[g]) * u;
}

// Source node of every far pair in group order: psrc[k] = far_src[svals[k]].
__global__ void k_pair_sources(int64_t nf, const int32_t* __restrict__ svals, const int32_t* __restrict__ far_src,
                               int32_t* __restrict__ psrc) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < nf) psrc[k] = far_src[svals[k]];
}

// Size in floats of a group's split operator (halves x chunks x (hi + lo) x
// 128 x KC).
__global__ void k_gop_sizes(int ng, const int32_t* __restrict__ gq, int64_t* __restrict__ sz) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > ng) return;
    if (g == ng) {
        sz[g] = 0;
        return;
    }
    const int q = gq[g], nrq = (q + 1) * (q + 1), nch = (nrq + kTcKC - 1) / kTcKC;
    sz[g] = (int64_t)tc_halves(q) * nch * 2 * kTcRows * kTcKC;
}

// Block per group: G_fs = a^(|f|+1) b^|s| T_{f+s}(D_c) split into TF32 parts,
// written half by half and chunk by chunk in the operand layout:
// [half][chunk][hi 128 x KC][lo 128 x KC] (half h: rows f = 128 h ..).
__global__ void __launch_bounds__(256) k_group_operator(int ldT, const float* __restrict__ gT,
                                                        const int32_t* __restrict__ gq,
                                                        const float2* __restrict__ gab,
                                                        const int64_t* __restrict__ goff, int g0, int64_t gop_base,
                                                        float* __restrict__ gop) {
    __shared__ int dec[(kMaxP + 1) * (kMaxP + 1)];
    __shared__ float apow[32], bpow[32];
    __shared__ float Tsh[1 + 3 * (2 * kMaxP) * (2 * kMaxP + 1) / 2];
    const int g = g0 + blockIdx.x;
    const int q = gq[g];
    const int nrq = (q + 1) * (q + 1), nch = (nrq + kTcKC - 1) / kTcKC, nrow = tc_halves(q) * kTcRows;
    for (int e = threadIdx.x; e < nrq; e += blockDim.x) dec[e] = qcomp(e);
    if (threadIdx.x < 32) {
        const float2 ab = gab[g];
        float a = 1.0f, b = 1.0f;
        for (int u = 0; u < (int)threadIdx.x; ++u) {
            a *= ab.x;
            b *= ab.y;
        }
        apow[threadIdx.x] = a;
        bpow[threadIdx.x] = b;
    }
    const int nTq = rbase(2 * q + 1);
    for (int e = threadIdx.x; e < nTq; e += blockDim.x) Tsh[e] = gT[(size_t)g * ldT + e];
    __syncthreads();
    float* out = gop + (goff[g] - gop_base);
    // consecutive threads write consecutive floats of a (half, chunk) block:
    // pos inverts tc_off(r, k) = (r/8) 64 + (k/4) 32 + (r%8) 4 + k%4
    constexpr int BLK = kTcRows * kTcKC;
    const int nblk = (nrow / kTcRows) * nch;
    for (int e = threadIdx.x; e < nblk * BLK; e += blockDim.x) {
        const int blk = e / BLK, pos = e - blk * BLK;
        const int half = blk / nch, ch = blk - half * nch;
        const int n = half * kTcRows + (pos >> 6) * 8 + ((pos & 31) >> 2);
        const int s = ch * kTcKC + ((pos >> 5) & 1) * 4 + (pos & 3);
        float v = 0.0f;
        if (n < nrq && s < nrq) {
            const int cs = dec[s], cf = dec[n];
            const int x = (cs & 0xff) + (cf & 0xff), y = ((cs >> 8) & 0xff) + ((cf >> 8) & 0xff),
                      z = ((cs >> 16) & 0xff) + ((cf >> 16) & 0xff);
            v = apow[(cf >> 24) + 1] * bpow[cs >> 24] * Tsh[ridx(x, y, z)];
        }
        float h, l;
        umma::split_tf32(v, h, l);
        float* o = out + (size_t)blk * 2 * BLK + pos;
        o[0] = h;
        o[BLK] = l;
    }
}

// Source nodes of a producer thread's rows 8 (rg0 + k * producer warps) + rsub of task t.
template <int RG>
__device__ __forceinline__ void tc_load_rows(int t, const int2* __restrict__ tasks, const int32_t* __restrict__ gstart,
                                             const int32_t* __restrict__ psrc, int rg0, int rsub, int (&r)[RG]) {
    const int2 tk = tasks[t];
    const int gs = gstart[tk.x] + (tk.y >> 1), cnt = min(kTcPairs, gstart[tk.x + 1] - gs);
#pragma unroll
    for (int k = 0; k < RG; ++k) {
        const int pr = 8 * (rg0 + (kTcProducers / 32) * k) + rsub;
        r[k] = pr < cnt ? psrc[gs + pr] : -1;
    }
}

__global__ void __launch_bounds__(kTcThreads, 1) k_m2l_tc(const int2* __restrict__ tasks, int ntasks,
                                                         const int32_t* __restrict__ gstart,
                                                         const int32_t* __restrict__ gq,
                                                         const int64_t* __restrict__ goff, int64_t gop_base,
                                                         const float* __restrict__ gop,
                                                         const int32_t* __restrict__ psrc,
                                                         const float* __restrict__ wsp, int ldk,
                                                         float* __restrict__ out,
                                                         const int32_t* __restrict__ rowbase,
                                                         int* __restrict__ err) {
    extern __shared__ __align__(1024) char sm_tc[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint64_t* full = reinterpret_cast<uint64_t*>(sm_tc + TcSmem::off_bar);
    uint64_t* empty = full + kTcStages;
    uint64_t* acc_full = empty + kTcStages;
    uint64_t* acc_empty = acc_full + 2;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm_tc + TcSmem::off_tmem);
    if (warp == 0) {
        umma::tmem_alloc(tslot, kTcCols);
        umma::tmem_relinquish();
    }
    if (tid == 0) {
        for (int st = 0; st < kTcStages; ++st) {
            umma::mbar_init(&full[st], kTcProducers + 1);  // producers' cp.async arrivals + the bulk copy's
            umma::mbar_init(&empty[st], 1);
        }
        for (int a = 0; a < 2; ++a) {
            umma::mbar_init(&acc_full[a], 1);
            umma::mbar_init(&acc_empty[a], kTcEpiWarps);  // one arrival per epilogue warp
        }
        umma::mbar_fence_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    bool ok = true;
    if (warp < kTcProducers / 32) {
        // ---- producers.  Each gather instruction covers one 8-row group x
        // (hi, lo) x two 16-byte pieces, which spreads its 512 bytes over all
        // shared-memory banks; a thread keeps its 16 rows' source nodes (-1:
        // no pair) in registers, loaded one task ahead.
        const int pt = tid, plane = tid & 31;
        const int part = plane >> 4, j = (plane >> 3) & 1, rsub = plane & 7;
        constexpr int RG = kTcPairs / 8 / (kTcProducers / 32);  // row groups per thread
        const int rg0 = pt >> 5;
        const uint64_t keep = umma::l2_evict_last();  // the weights stay in L2 beside the result stream
        uint32_t u = 0;
        int task = blockIdx.x;
        int rows[RG], nrows[RG];
        if (task < ntasks) tc_load_rows<RG>(task, tasks, gstart, psrc, rg0, rsub, rows);
        while (task < ntasks && ok) {
            const int g = tasks[task].x, q = gq[g];
            const int nch = ((q + 1) * (q + 1) + kTcKC - 1) / kTcKC;
            const int next = task + gridDim.x;
            if (next < ntasks) tc_load_rows<RG>(next, tasks, gstart, psrc, rg0, rsub, nrows);  // in flight
            // the task's operator half
            const float* G = gop + (goff[g] - gop_base) + (size_t)(tasks[task].y & 1) * nch * 2 * TcSmem::g_floats;
            for (int ch = 0; ch < nch; ++ch, ++u) {
                const int st = (int)(u % kTcStages);
                if (u >= (uint32_t)kTcStages &&
                    !umma::mbar_wait(&empty[st], ((u / kTcStages) - 1) & 1, kTcWaitCycles)) {
                    ok = false;
                    break;
                }
                float* Gs = reinterpret_cast<float*>(sm_tc + (size_t)st * TcSmem::stage_bytes);
                float* Ws = Gs + 2 * TcSmem::g_floats;
                if (pt == 0) {
                    constexpr uint32_t gb = sizeof(float) * 2 * TcSmem::g_floats;
                    umma::mbar_arrive_expect_tx(&full[st], gb);
                    umma::bulk_g2s(Gs, G + (size_t)ch * 2 * TcSmem::g_floats, gb, &full[st]);
                }
                float* dst0 = Ws + part * TcSmem::w_floats + 4 * j * 8 + rsub * 4;  // tc_off(8 rg + rsub, 4 j)
                const int coff = ch * 2 * kTcKC + part * kTcKC + 4 * j;
#pragma unroll
                for (int k = 0; k < RG; ++k) {
                    const int src = rows[k];
                    const float* gsrc = src >= 0 ? wsp + (size_t)src * 2 * ldk + coff : wsp;
                    umma::cp16_keep(dst0 + (rg0 + (kTcProducers / 32) * k) * kTcKC * 8, gsrc, src >= 0, keep);
                }
                umma::cp_async_mbar_arrive(&full[st]);
            }
#pragma unroll
            for (int k = 0; k < RG; ++k) rows[k] = nrows[k];
            task = next;
        }
    } else if (warp == kTcMmaWarp) {
        // ---- MMA issue (one thread)
        if (lane == 0) {
            uint32_t u = 0, tl = 0;
            const uint32_t idesc = umma::idesc_tf32(kTcRows, kTcPairs);
            constexpr uint32_t LBO = 128, SBO = kTcKC / 4 * 128;
            for (int task = blockIdx.x; task < ntasks && ok; task += gridDim.x) {
                const int g = tasks[task].x, q = gq[g];
                const int nch = ((q + 1) * (q + 1) + kTcKC - 1) / kTcKC;
                const int acc = (int)(tl & 1);
                if (tl >= 2 && !umma::mbar_wait(&acc_empty[acc], ((tl >> 1) - 1) & 1, kTcWaitCycles)) {
                    ok = false;
                    break;
                }
                umma::fence_after_sync();
                const uint32_t d = tmem + (uint32_t)(acc * kTcPairs);
                for (int ch = 0; ch < nch; ++ch, ++u) {
                    const int st = (int)(u % kTcStages);
                    if (!umma::mbar_wait(&full[st], (u / kTcStages) & 1, kTcWaitCycles)) {
                        ok = false;
                        break;
                    }
                    umma::fence_proxy_async();  // the cp.async data, for the tensor cores
                    umma::fence_after_sync();
                    const float* Gs = reinterpret_cast<const float*>(sm_tc + (size_t)st * TcSmem::stage_bytes);
                    const float* Ws = Gs + 2 * TcSmem::g_floats;
                    const uint64_t gh = umma::smem_desc(Gs, LBO, SBO);
                    const uint64_t gl = umma::smem_desc(Gs + TcSmem::g_floats, LBO, SBO);
                    const uint64_t wh = umma::smem_desc(Ws, LBO, SBO);
                    const uint64_t wl = umma::smem_desc(Ws + TcSmem::w_floats, LBO, SBO);
                    umma::mma_tf32(d, gh, wh, idesc, ch > 0 ? 1u : 0u);
                    umma::mma_tf32(d, gh, wl, idesc, 1u);
                    umma::mma_tf32(d, gl, wh, idesc, 1u);
                    umma::commit(&empty[st]);
                }
                if (!ok) break;
                umma::commit(&acc_full[acc]);
                ++tl;
            }
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. + 31
        // (with more than four epilogue warps, each of a sub-partition's warps
        // takes its share of the columns), kTcEpiBatch loads per wait
        const int sp = warp & 3;
        const int f = 32 * sp + lane;
        constexpr int kShares = kTcEpiWarps / 4;
        const int share = (warp - 3) / 4;
        constexpr int CB = 16 * kTcEpiBatch;  // columns per wait
        uint32_t tl = 0;
        for (int task = blockIdx.x; task < ntasks && ok; task += gridDim.x) {
            const int2 tk = tasks[task];
            const int g = tk.x, q = gq[g];
            const int f0 = kTcRows * (tk.y & 1), fr = f0 + f;  // the task's operator half; this lane's row
            const int gs = gstart[g] + (tk.y >> 1);
            const int cnt = min(kTcPairs, gstart[g + 1] - gs);
            const int acc = (int)(tl & 1);
            if (!umma::mbar_wait(&acc_full[acc], (tl >> 1) & 1, kTcWaitCycles)) {
                ok = false;
                break;
            }
            umma::fence_after_sync();
            const uint32_t base = tmem + ((uint32_t)(32 * sp) << 16) + (uint32_t)(acc * kTcPairs);
            // the group's rows: (q+1)^2 rounded up to kRowUnit entries, from
            // rowbase[g] x kRowUnit in group order
            const int rl = row_len(q);
            float* gout = out + ((size_t)rowbase[g] + (size_t)(tk.y >> 1) * (rl / kRowUnit)) * kRowUnit;
            // warps whose 32 rows f lie beyond the row length have nothing to write
#pragma unroll 1
            for (int c = share * CB; c < cnt && f0 + 32 * sp < rl; c += kShares * CB) {
                float v[CB];
#pragma unroll
                for (int b = 0; b < kTcEpiBatch; ++b) umma::tmem_ld16(base + (uint32_t)(c + 16 * b), v + 16 * b);
                umma::tmem_ld_wait();
                // the task's rows are consecutive; streaming stores of whole lines
                if (fr < rl) {
#pragma unroll
                    for (int jj = 0; jj < CB; ++jj)
                        if (c + jj < cnt) __stcs(gout + (size_t)(c + jj) * rl + fr, v[jj]);
                }
            }
            umma::fence_before_sync();
            __syncwarp();
            if (lane == 0) umma::mbar_arrive(&acc_empty[acc]);
            ++tl;
        }
    }
    if (!ok) atomicExch(err, 1);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, kTcCols);
}

// Running sum of one output: FP32 values as a double-float pair (TwoSum, on
// the FP32 pipe), FP64 values in FP64.
template <typename R>
struct Sum;
template <>
struct Sum<float> {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float s = hi + v;
        const float bb = s - hi;
        lo += (hi - (s - bb)) + (v - bb);
        hi = s;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
template <>
struct Sum<double> {
    double v = 0.0;
    __device__ __forceinline__ void add(double x) { v += x; }
    __device__ __forceinline__ double value() const { return v; }
};

// Block per target, thread per reduced component: compensated sum of the
// target's pair rows (stored in group order; roff gives each target-order
// pair's row in units of kRowUnit entries; a pair of order q contributes its first
// (q+1)^2 entries; eight loads in flight), back to physical units, into the
// reduced components of the local expansion.
template <typename R>
__global__ void __launch_bounds__(256) k_m2l_sum(const TreeDev t, int p, const R* __restrict__ out,
                                                 const int32_t* __restrict__ roff, double* __restrict__ loc) {
    const int i = blockIdx.x;
    const int nr = (p + 1) * (p + 1);
    const int q0 = t.far_off[i], q1 = t.far_off[i + 1];
    const double ih = 1.0 / t.r[i];
    double* L = loc + (size_t)i * nT(p);
    for (int f = threadIdx.x; f < nr; f += blockDim.x) {
        constexpr int U = 8;
        Sum<R> acc;
        int q = q0;
        for (; q + U <= q1; q += U) {
            R v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int qq = t.far_ord ? min((int)t.far_ord[q + u], p) : p;
                v[u] = f < (qq + 1) * (qq + 1) ? out[(size_t)roff[q + u] * kRowUnit + f] : (R)0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) acc.add(v[u]);
        }
        for (; q < q1; ++q) {
            const int qq = t.far_ord ? min((int)t.far_ord[q], p) : p;
            if (f < (qq + 1) * (qq + 1)) acc.add(out[(size_t)roff[q] * kRowUnit + f]);
        }
        const int c = qcomp(f);
        const int k = c >> 24;
        double s = ih;
        for (int e = 0; e < k; ++e) s *= ih;
        L[pidx(c & 0xff, (c >> 8) & 0xff, (c >> 16) & 0xff)] = acc.value() * s;
    }
}

// FP32 products on the CUDA cores instead of the tensor cores
// (FMM_GB300_M2L_PRODUCT=cuda; read at every call).
bool product_on_cuda_cores() {
    const char* e = std::getenv("FMM_GB300_M2L_PRODUCT");
    return e && std::strcmp(e, "cuda") == 0;
}

// Orders share a displacement group in classes of kOrderClass consecutive
// orders; the group takes its pairs' highest order (fewer operators for the
// learned selector's mixed orders).
constexpr int kOrderClass = 2;

constexpr double kMinGroupPairs = 16.0;    // mean far pairs per displacement group for the grouped products
constexpr double kOperatorBytes = 16e9;  // TF32 operator parts of one batch of groups

template <typename R, int CPT>
int grouped(Workspace& ws, const TreeDev& t, int p, cudaStream_t st) {
    const int M = t.num_nodes, nr = (p + 1) * (p + 1), N = 2 * p, nTr = rbase(N + 1);
    const bool tc = sizeof(R) == 4 && !product_on_cuda_cores();
    const int cols = tc ? -1 : kTaskCols;  // -1: tensor-core tasks (256 pairs, one operator half)
    const int64_t nf = t.nfar;
    const int ldw = wsc_ld<R>(nr);
    const int ldk = (nr + 15) / 16 * 16;
    const int ldT = nTr;
    const int32_t* roff = nullptr;  // row of each far pair (target order), units of 32 entries
    if (nf > 0 && !ws.reuse_structure) {
        // structure: displacement groups, their tensors and operators, tasks
        // and result rows (geometry only; kept for replays)
        ws.m2l_pairwise = false;
        FMM_TRY(ws.m2l_tgt.ensure(sizeof(int32_t) * nf));
        FMM_TRY(ws.m2l_keys.ensure(sizeof(uint64_t) * nf));
        FMM_TRY(ws.m2l_keys2.ensure(sizeof(uint64_t) * nf));
        FMM_TRY(ws.m2l_vals.ensure(sizeof(int32_t) * nf));
        FMM_TRY(ws.m2l_vals2.ensure(sizeof(int32_t) * nf));
        FMM_TRY(ws.m2l_ukeys.ensure(sizeof(uint64_t) * nf));
        FMM_TRY(ws.m2l_cnt.ensure(sizeof(int32_t) * (nf + 1)));
        FMM_TRY(ws.m2l_gstart.ensure(sizeof(int32_t) * (nf + 1)));
        FMM_TRY(ws.m2l_wsc.ensure(sizeof(R) * (size_t)M * ldw));
        FMM_TRY(ws.counters.ensure(sizeof(unsigned long long) * 32));
        int32_t* tgt = ws.m2l_tgt.as<int32_t>();
        count_launches(1);
        k_far_targets<<<grid_for(M, 4), 128, 0, st>>>(M, t.far_off, tgt);
        count_launches(1);
        // FP32 node data where the mixed path prepared it
        const float4* chi = (sizeof(R) == 4 && ws.f32node_ok) ? ws.f32node.as<float4>() : nullptr;
        k_m2l_keys<<<grid_for(nf, 256), 256, 0, st>>>(nf, t, tgt, p, kOrderClass, chi, chi ? chi + M : nullptr,
                                                       ws.m2l_keys.as<uint64_t>(), ws.m2l_vals.as<int32_t>());
        // sort by key, run-length encode into groups
        int* d_nruns = reinterpret_cast<int*>(ws.counters.as<unsigned long long>() + 14);
        size_t tb1 = 0, tb2 = 0, tb3 = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tb1, ws.m2l_keys.as<uint64_t>(), ws.m2l_keys2.as<uint64_t>(),
                                        ws.m2l_vals.as<int32_t>(), ws.m2l_vals2.as<int32_t>(), (int)nf, 0, kKeyBits, st);
        cub::DeviceRunLengthEncode::Encode(nullptr, tb2, ws.m2l_keys2.as<uint64_t>(), ws.m2l_ukeys.as<uint64_t>(),
                                           ws.m2l_cnt.as<int32_t>(), d_nruns, (int)nf, st);
        cub::DeviceScan::ExclusiveSum(nullptr, tb3, ws.m2l_cnt.as<int32_t>(), ws.m2l_gstart.as<int32_t>(),
                                      (int)nf + 1, st);
        FMM_TRY(ws.cub_tmp.ensure(std::max(tb1, std::max(tb2, tb3))));
        FMM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(ws.cub_tmp.p, tb1, ws.m2l_keys.as<uint64_t>(),
                                                     ws.m2l_keys2.as<uint64_t>(), ws.m2l_vals.as<int32_t>(),
                                                     ws.m2l_vals2.as<int32_t>(), (int)nf, 0, kKeyBits, st));
        FMM_CUDA_TRY(cub::DeviceRunLengthEncode::Encode(ws.cub_tmp.p, tb2, ws.m2l_keys2.as<uint64_t>(),
                                                        ws.m2l_ukeys.as<uint64_t>(), ws.m2l_cnt.as<int32_t>(),
                                                        d_nruns, (int)nf, st));
        int ng = 0;
        FMM_CUDA_TRY(cudaMemcpyAsync(&ng, d_nruns, sizeof(int), cudaMemcpyDeviceToHost, st));
        FMM_CUDA_TRY(cudaStreamSynchronize(st));
        ws.m2l_groups = ng;
        // displacement groups of a few pairs each (irregular trees, mixed
        // orders) leave the products' columns empty and multiply the
        // per-group operators: the per-pair kernel is then the faster one
        if ((double)nf < kMinGroupPairs * (double)ng) {
            ws.m2l_pairwise = true;
            return FMM_ENOTSUP;
        }
        FMM_CUDA_TRY(cudaMemsetAsync(ws.m2l_cnt.as<int32_t>() + ng, 0, sizeof(int32_t), st));
        size_t tb4 = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb4, ws.m2l_cnt.as<int32_t>(), ws.m2l_gstart.as<int32_t>(), ng + 1, st);
        FMM_TRY(ws.cub_tmp.ensure(tb4));
        FMM_CUDA_TRY(cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tb4, ws.m2l_cnt.as<int32_t>(),
                                                   ws.m2l_gstart.as<int32_t>(), ng + 1, st));
        // per-group tensors
        FMM_TRY(ws.m2l_T.ensure(sizeof(R) * (size_t)ng * ldT));
        FMM_TRY(ws.m2l_gq.ensure(sizeof(int32_t) * ng));
        FMM_TRY(ws.m2l_gab.ensure(sizeof(float2) * ng));
        {
            const int wpb = 4;
            const size_t sm = sizeof(double) * (nTr + (size_t)wpb * (2 * nTr + N + 1));
            if (sm > 48 * 1024)
                FMM_CUDA_TRY(cudaFuncSetAttribute((const void*)k_group_tensor<R>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            count_launches(1);
            k_group_tensor<R><<<grid_for(ng, wpb), 32 * wpb, sm, st>>>(
                ng, ws.m2l_ukeys.as<uint64_t>(), ws.m2l_gstart.as<int32_t>(), ws.m2l_vals2.as<int32_t>(), tgt, t, p,
                ldT, ws.m2l_T.as<R>(), ws.m2l_gq.as<int32_t>(), ws.m2l_gab.as<float2>());
        }
        // tasks: up to kTaskCols pairs of one group each (tensor cores: 256
        // pairs and one operator half)
        FMM_TRY(ws.m2l_tcnt.ensure(sizeof(int32_t) * (ng + 1)));
        FMM_TRY(ws.m2l_toff.ensure(sizeof(int32_t) * (ng + 1)));
        count_launches(1);
        k_task_counts<<<grid_for(ng + 1, 256), 256, 0, st>>>(ng, cols, ws.m2l_gq.as<int32_t>(),
                                                              ws.m2l_gstart.as<int32_t>(), ws.m2l_tcnt.as<int32_t>());
        size_t tb5 = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb5, ws.m2l_tcnt.as<int32_t>(), ws.m2l_toff.as<int32_t>(), ng + 1, st);
        FMM_TRY(ws.cub_tmp.ensure(tb5));
        FMM_CUDA_TRY(cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tb5, ws.m2l_tcnt.as<int32_t>(),
                                                   ws.m2l_toff.as<int32_t>(), ng + 1, st));
        // result rows in group order, (q+1)^2 rounded up to kRowUnit entries per
        // pair; the per-target sum finds them through roff (in the free
        // unsorted-keys buffer)
        FMM_TRY(ws.m2l_rowbase.ensure(sizeof(int32_t) * (ng + 1)));
        int32_t* rowbase = ws.m2l_rowbase.as<int32_t>();
        count_launches(1);
        k_row_sizes<<<grid_for(ng + 1, 256), 256, 0, st>>>(ng, ws.m2l_gstart.as<int32_t>(), ws.m2l_gq.as<int32_t>(),
                                                            rowbase);
        size_t tb7 = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb7, rowbase, rowbase, ng + 1, st);
        FMM_TRY(ws.cub_tmp.ensure(tb7));
        FMM_CUDA_TRY(cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tb7, rowbase, rowbase, ng + 1, st));
        count_launches(1);
        k_row_offsets<<<grid_for(ng, 8), 256, 0, st>>>(ng, ws.m2l_gstart.as<int32_t>(), ws.m2l_gq.as<int32_t>(),
                                                        rowbase, ws.m2l_vals2.as<int32_t>(),
                                                        reinterpret_cast<int32_t*>(ws.m2l_keys.p));
        int hcnt[2] = {0, 0};  // tasks, rows (units of 32 entries)
        FMM_CUDA_TRY(cudaMemcpyAsync(&hcnt[0], ws.m2l_toff.as<int32_t>() + ng, sizeof(int), cudaMemcpyDeviceToHost, st));
        FMM_CUDA_TRY(cudaMemcpyAsync(&hcnt[1], rowbase + ng, sizeof(int), cudaMemcpyDeviceToHost, st));
        FMM_CUDA_TRY(cudaStreamSynchronize(st));
        const int ntasks = hcnt[0];
        FMM_TRY(ws.m2l_out.ensure(sizeof(R) * kRowUnit * (size_t)std::max(1, hcnt[1])));
        FMM_TRY(ws.m2l_tasks.ensure(sizeof(int2) * std::max(1, ntasks)));
        count_launches(1);
        k_fill_tasks<<<grid_for(ng, 256), 256, 0, st>>>(ng, cols, ws.m2l_gq.as<int32_t>(), ws.m2l_gstart.as<int32_t>(),
                                                        ws.m2l_toff.as<int32_t>(), ws.m2l_tasks.as<int2>());
        if (tc) {
            FMM_TRY(ws.m2l_wsplit.ensure(sizeof(float) * 2 * (size_t)M * ldk));
            // source node per sorted pair (into the free unsorted-values buffer)
            count_launches(1);
            k_pair_sources<<<grid_for(nf, 256), 256, 0, st>>>(nf, ws.m2l_vals2.as<int32_t>(), t.far_src,
                                                              ws.m2l_vals.as<int32_t>());
            FMM_TRY(ws.m2l_gopoff.ensure(sizeof(int64_t) * (ng + 1)));
            int64_t* goff = ws.m2l_gopoff.as<int64_t>();
            count_launches(1);
            k_gop_sizes<<<grid_for(ng + 1, 256), 256, 0, st>>>(ng, ws.m2l_gq.as<int32_t>(), goff);
            size_t tb6 = 0;
            cub::DeviceScan::ExclusiveSum(nullptr, tb6, goff, goff, ng + 1, st);
            FMM_TRY(ws.cub_tmp.ensure(tb6));
            FMM_CUDA_TRY(cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tb6, goff, goff, ng + 1, st));
            // TF32 parts of the operators (per group, at each group's order),
            // in batches of consecutive groups of at most kOperatorBytes: one
            // batch is built here once; several are built, each before the
            // product over its tasks, at every evaluation
            std::vector<int64_t> hgoff((size_t)ng + 1);
            std::vector<int32_t> htoff((size_t)ng + 1);
            FMM_CUDA_TRY(cudaMemcpyAsync(hgoff.data(), goff, sizeof(int64_t) * (ng + 1), cudaMemcpyDeviceToHost, st));
            FMM_CUDA_TRY(cudaMemcpyAsync(htoff.data(), ws.m2l_toff.as<int32_t>(), sizeof(int32_t) * (ng + 1),
                                         cudaMemcpyDeviceToHost, st));
            FMM_CUDA_TRY(cudaStreamSynchronize(st));
            const int64_t cap = (int64_t)(kOperatorBytes / sizeof(float));
            ws.m2l_batches.clear();
            int64_t biggest = 0;
            for (int g0 = 0; g0 < ng;) {
                int g1 = g0 + 1;
                while (g1 < ng && hgoff[g1 + 1] - hgoff[g0] <= cap) ++g1;
                ws.m2l_batches.push_back({g0, g1, hgoff[g0], htoff[g0], htoff[g1]});
                biggest = std::max(biggest, hgoff[g1] - hgoff[g0]);
                g0 = g1;
            }
            FMM_TRY(ws.m2l_gop.ensure(sizeof(float) * std::max<int64_t>(1, biggest)));
            if (ws.m2l_batches.size() == 1) {
                count_launches(1);
                k_group_operator<<<(unsigned)ng, 256, 0, st>>>(ldT, reinterpret_cast<const float*>(ws.m2l_T.p),
                                                               ws.m2l_gq.as<int32_t>(), ws.m2l_gab.as<float2>(), goff,
                                                               0, 0, ws.m2l_gop.as<float>());
            }
        }
        ws.m2l_ng = ng;
        ws.m2l_ntasks = ntasks;
    }
    if (nf > 0) {
        // numeric: scaled weights, the product, (below) the per-target sums
        const int ntasks = ws.m2l_ntasks;
        const int32_t* rowbase = ws.m2l_rowbase.as<int32_t>();
        roff = reinterpret_cast<const int32_t*>(ws.m2l_keys.p);
        count_launches(1);
        k_scale_weights<R><<<grid_for(M, 4), 128, 0, st>>>(M, nr, ldw, ws.wred.as<double>(), t.r, ws.m2l_wsc.as<R>());
        int* d_err = reinterpret_cast<int*>(ws.counters.as<unsigned long long>() + 13);
        if (tc) {
            // TF32 parts of the weights (per node)
            count_launches(1);
            k_split_weights<<<grid_for((int64_t)M * ldk, 256), 256, 0, st>>>(
                (int64_t)M * ldk, nr, ldw, ldk, reinterpret_cast<const float*>(ws.m2l_wsc.p), ws.m2l_wsplit.as<float>());
            FMM_CUDA_TRY(cudaFuncSetAttribute((const void*)k_m2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)TcSmem::bytes));
            int dev = 0, sms = 0;
            FMM_CUDA_TRY(cudaGetDevice(&dev));
            FMM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            if (!ws.product_err) FMM_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));  // first product of the call
            if (ws.events_ready) {
                cudaEventRecord(ws.ev[8], st);
                ws.product_timed = true;
            }
            const bool many = ws.m2l_batches.size() > 1;
            for (const M2lBatch& b : ws.m2l_batches) {
                if (many) {
                    count_launches(1);
                    k_group_operator<<<(unsigned)(b.g1 - b.g0), 256, 0, st>>>(
                        ldT, reinterpret_cast<const float*>(ws.m2l_T.p), ws.m2l_gq.as<int32_t>(),
                        ws.m2l_gab.as<float2>(), ws.m2l_gopoff.as<int64_t>(), b.g0, b.gop_base, ws.m2l_gop.as<float>());
                }
                const int nt = b.t1 - b.t0;
                if (nt <= 0) continue;
                const int grid = std::max(1, std::min(nt, sms));  // one block per SM (all tensor memory)
                count_launches(1);
                k_m2l_tc<<<(unsigned)grid, kTcThreads, TcSmem::bytes, st>>>(
                    ws.m2l_tasks.as<int2>() + b.t0, nt, ws.m2l_gstart.as<int32_t>(), ws.m2l_gq.as<int32_t>(),
                    ws.m2l_gopoff.as<int64_t>(), many ? b.gop_base : 0, ws.m2l_gop.as<float>(),
                    ws.m2l_vals.as<int32_t>(), ws.m2l_wsplit.as<float>(), ldk, reinterpret_cast<float*>(ws.m2l_out.p),
                    rowbase, d_err);
            }
            if (ws.product_timed) cudaEventRecord(ws.ev[9], st);
            // the product's error flag is read with the call's final copies
            ws.product_err = d_err;
        } else {
            const GemmSmem<R, CPT> L(p);
            FMM_CUDA_TRY(cudaFuncSetAttribute((const void*)k_m2l_gemm<R, CPT>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.bytes));
            if (ws.events_ready) {
                cudaEventRecord(ws.ev[8], st);
                ws.product_timed = true;
            }
            count_launches(1);
            k_m2l_gemm<R, CPT><<<(unsigned)ntasks, kGemmThreads, L.bytes, st>>>(
                ws.m2l_tasks.as<int2>(), cols, 0, p, ws.m2l_gstart.as<int32_t>(), ws.m2l_gq.as<int32_t>(),
                ws.m2l_gab.as<float2>(), ws.m2l_T.as<R>(), ldT, ws.m2l_vals2.as<int32_t>(), t.far_src,
                ws.m2l_wsc.as<R>(), ws.m2l_out.as<R>(), rowbase);
            if (ws.product_timed) cudaEventRecord(ws.ev[9], st);
        }
    }
    count_launches(1);
    if (nf == 0) FMM_TRY(ws.m2l_out.ensure(sizeof(R) * kRowUnit));
    // one output per thread: (p+1)^2 rounded up to whole warps (192 at p = 12)
    k_m2l_sum<R><<<(unsigned)M, (unsigned)std::min(256, (nr + 31) / 32 * 32), 0, st>>>(t, p, ws.m2l_out.as<R>(), roff,
                                                                                     ws.loc.as<double>());
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace

// Grouped reduced-basis M2L into the reduced components of ws.loc (the
// weights ws.wred must be current).  FP32 products for `fp32`, else FP64;
// returns FMM_ENOTSUP where the FP64 operator does not fit shared memory.
int launch_m2l_grouped(Workspace& ws, const TreeDev& t, int p, bool fp32, cudaStream_t st) {
    if (fp32) return grouped<float, 8>(ws, t, p, st);
    if (GemmSmem<double, 4>(p).bytes > 227 * 1024) return FMM_ENOTSUP;
    return grouped<double, 4>(ws, t, p, st);
}

}  // namespace fmm

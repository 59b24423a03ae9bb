// Mixed-precision near field (P2P): FP32 pair arithmetic with FP64 sums.
//
// Same pairs as particle_fields (src/fmm.F90:623-747).  Coordinates are held
// in FP32 relative to each particle's own leaf centre; for a target leaf A and
// a source leaf B the displacement is
//     R = (x_t - x_s) + (c_A - c_B),
// with the centre offset formed in FP64 once per leaf pair, so the FP32
// rounding error scales with the leaf size and |R|, not with the distance from
// the box origin.  Positions are double-float pairs, r^2 is compensated and
// 1/r Newton-refined.  Contributions are summed over one source leaf in
// compensated FP32 (TwoSum hi + lo) and the per-leaf sums are added into FP64
// accumulators.  Excluded partners and the self pair are masked in the loop.
//
// The packed kernel (field orders 0 and 1, all kernels but erf) evaluates
// each target against two sources at once in f32x2 arithmetic from a second
// record array with even leaf starts and interleaved slot pairs, and, with
// learned lists on AMOEBA, walks a damping-correction list after the near
// list: far leaf pairs inside the damping range, of which only the pairs
// with a r below the range's cutoff are evaluated, as the difference of the
// damped and undamped kernels (the M2L carries the undamped one).
#include <algorithm>
#include <cstdlib>

#include <cub/cub.cuh>

#include "dispatch.cuh"
#include "internal.h"
#include "pair.cuh"
#include "pair_x2.cuh"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

constexpr int kExwRegs = 8;  // exclusion entries held in registers per target

// Sub-chunks of a target leaf's last rem < 32 particles (index rem): the
// count that minimises the lane-steps of a piece of source blocks for leaves
// of about 30 particles (c sub-chunks of ceil(rem / c) targets run
// floor(32 / ceil(rem / c)) lane groups each).
__constant__ int kSubChunks[32] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 1, 1, 1,
                                   1, 3, 3, 2, 2, 3, 3, 3, 3, 1, 1, 1, 1, 1, 1, 1};

// Per sorted particle, one record of float4s: (x, y, z, d), (x_lo, y_lo, z_lo,
// original index + 1 as int bits), then the FP32 scaled multipoles padded to
// a multiple of 4 (for quadrupoles the first pad slot holds the trace of the
// scaled second moments, used by the near-field contraction).  Positions are relative to the particle's own leaf centre
// as double-float pairs (hi = rounded value, lo = rounded remainder), so
// differences of positions in two leaves lose nothing beyond the final FP32
// rounding.  A source is then read with a handful of 16-byte loads from one
// base address.
__host__ __device__ constexpr int rec_vec(int dim) { return 2 + (dim + 3) / 4; }

__global__ void k_gather_f32(int64_t n, int dim, const TreeDev t, const double* __restrict__ sx,
                             const double* __restrict__ sy, const double* __restrict__ sz,
                             const double* __restrict__ sd, const double* __restrict__ smc,
                             float4* __restrict__ rec) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int nv = rec_vec(dim);
    const int leaf = t.leaf_of[k];
    const double rx = sx[k] - t.cx[leaf], ry = sy[k] - t.cy[leaf], rz = sz[k] - t.cz[leaf];
    const float hx = (float)rx, hy = (float)ry, hz = (float)rz;
    float4* r = rec + (size_t)k * nv;
    r[0] = make_float4(hx, hy, hz, (float)sd[k]);
    r[1] = make_float4((float)(rx - (double)hx), (float)(ry - (double)hy), (float)(rz - (double)hz),
                       __int_as_float((int32_t)t.perm[k] + 1));  // 1-based, as in the exclusion lists
    for (int v = 2; v < nv; ++v) {
        float m[4];
        for (int c = 0; c < 4; ++c) {
            const int s = 4 * (v - 2) + c;
            m[c] = s < dim ? (float)smc[(size_t)s * n + k] : 0.0f;
            if (dim == 10 && s == 10)
                m[c] = (float)(smc[(size_t)4 * n + k] + smc[(size_t)7 * n + k] + smc[(size_t)9 * n + k]);
        }
        r[v] = make_float4(m[0], m[1], m[2], m[3]);
    }
}

// Source records of the packed near field: the sorted particles of each leaf
// from an even slot ps[leaf] on, an odd leaf padded by one empty particle
// (zero multipoles, 1000 bohr from its leaf centre, damping factor 1: its
// pair terms are exactly zero); slots 2b and 2b + 1 form block b, stored
// element by element interleaved (float 2e + h of the block is element e of
// the record of slot 2b + h), so one 16-byte shared-memory load gives two
// elements of both particles as two packed pairs.
// With q1 (quadrupole sources, field order 1: contract_q1_x2) the
// off-diagonal second moments xy, xz, yz (record elements 13, 14, 16) are
// stored halved, an exact scaling.
__global__ void k_gather_x2(int64_t n, int nv, bool q1, const TreeDev t, const int32_t* __restrict__ ps,
                            const float4* __restrict__ rec, float* __restrict__ x2) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int leaf = t.leaf_of[k];
    const int within = (int)(k - t.start[leaf]), cnt = t.count[leaf];
    const int64_t slot = (int64_t)ps[leaf] + within;
    const float* s = reinterpret_cast<const float*>(rec + (size_t)k * nv);
    float* d = x2 + (size_t)(slot >> 1) * 8 * nv + (slot & 1);
    for (int e = 0; e < 4 * nv; ++e) d[2 * e] = s[e];
    if (q1) {
        d[2 * 13] = 0.5f * s[13];
        d[2 * 14] = 0.5f * s[14];
        d[2 * 16] = 0.5f * s[16];
    }
    if (within == cnt - 1 && (cnt & 1)) {
        float* dd = d + 1;  // slot + 1: the odd half of the same block
        for (int e = 0; e < 4 * nv; ++e) dd[2 * e] = 0.0f;
        dd[0] = 1000.0f;  // x
        dd[2 * 3] = 1.0f; // damping factor
    }
}

// Per leaf: the largest distance of its particles from its centre (from the
// FP32 records, plus a rounding margin) and its smallest damping factor;
// bounds for skipping whole damping-correction pieces.
__global__ void k_leaf_extent(int nv, const TreeDev t, const float4* __restrict__ rec, float2* __restrict__ ext) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= t.num_leaves) return;
    const int leaf = t.leaves[w];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    float r2 = 0.0f, dmin = 3.0e38f;
    for (int k = lane; k < cnt; k += 32) {
        const float4 a = rec[(size_t)(s0 + k) * nv];
        r2 = fmaxf(r2, a.x * a.x + a.y * a.y + a.z * a.z);
        dmin = fminf(dmin, a.w);
    }
    for (int o = 16; o > 0; o >>= 1) {
        r2 = fmaxf(r2, __shfl_xor_sync(0xffffffffu, r2, o));
        dmin = fminf(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    }
    if (lane == 0) ext[leaf] = make_float2(sqrtf(r2) * 1.0001f + 1e-3f, dmin);
}

__global__ void k_leaf_odd(const TreeDev t, int32_t* __restrict__ odd) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < t.num_leaves) odd[w] = t.count[t.leaves[w]] & 1;
}

// Leaves are in DFS order, i.e. by increasing start: the padded start of a
// leaf is its start plus the odd leaves before it.
__global__ void k_leaf_pstart(const TreeDev t, const int32_t* __restrict__ pre, int32_t* __restrict__ ps) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < t.num_leaves) ps[t.leaves[w]] = t.start[t.leaves[w]] + pre[w];
}

// Node centres as double-float pairs (hi = rounded centre, lo = rounded
// remainder), so leaf-centre offsets are formed in FP32 without losing bits;
// the w components carry rmax (hi) and the half-width (lo) in FP32 for the
// learned list build.
__global__ void k_node_centres_f32(int M, const TreeDev t, float4* __restrict__ hi, float4* __restrict__ lo) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    const float hx = (float)t.cx[k], hy = (float)t.cy[k], hz = (float)t.cz[k];
    hi[k] = make_float4(hx, hy, hz, (float)t.rmax[k]);
    lo[k] = make_float4((float)(t.cx[k] - (double)hx), (float)(t.cy[k] - (double)hy), (float)(t.cz[k] - (double)hz),
                        (float)t.r[k]);
}

// a - b as an unevaluated pair s + e (Knuth's TwoSum with b negated).
__device__ __forceinline__ float two_diff(float a, float b, float& e) {
    const float s = a - b;
    const float bb = s - a;
    e = (a - (s - bb)) - (b + bb);
    return s;
}

// FP32 field estimate at a few targets over all sources (exclusions masked),
// from the sorted FP32 records; only a magnitude is wanted (the learned
// selector's error budget).  Block per (target, source split); block sums
// added into out (ntgt x nF, column-major, zeroed by the caller).
template <int M, int F>
__global__ void __launch_bounds__(128) k_direct_scale(const TreeDev t, const float4* __restrict__ rec,
                                                      const float4* __restrict__ chi,
                                                      const int64_t* __restrict__ targets, int64_t ntgt, int64_t n,
                                                      int damp, int exw, const int32_t* __restrict__ excl,
                                                      int64_t chunk, double* __restrict__ out) {
    constexpr int NF = nT(F), NM = nT(M), NV = rec_vec(NM);
    __shared__ float red[NF][4];
    const int64_t ti = blockIdx.x;
    const int64_t i = targets[ti];
    const int it = t.pos_of[i];
    const float4 ta = rec[(size_t)it * NV], ca = chi[t.leaf_of[it]];
    const float tx = ta.x + ca.x, ty = ta.y + ca.y, tz = ta.z + ca.z;
    float acc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) acc[f] = 0.0f;
    const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    for (int64_t k = j0 + threadIdx.x; k < j1; k += blockDim.x) {
        if (k == it) continue;
        const float4* r = rec + (size_t)k * NV;
        const float4 sa = r[0], sb = r[1];
        const int o = __float_as_int(sb.w);
        bool ex = false;
        for (int e = 0; e < exw; ++e) ex |= (excl[(size_t)e * n + i] == o);
        if (ex) continue;
        const float4 cb = chi[t.leaf_of[k]];
        float mc[4 * (NV - 2)];
#pragma unroll
        for (int v = 0; v < NV - 2; ++v) {
            const float4 w = r[2 + v];
            mc[4 * v] = w.x;
            mc[4 * v + 1] = w.y;
            mc[4 * v + 2] = w.z;
            mc[4 * v + 3] = w.w;
        }
        pair_field<M, F, float>(tx - (sa.x + cb.x), ty - (sa.y + cb.y), tz - (sa.z + cb.z), ta.w * sa.w, damp, mc,
                                acc);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        float v = acc[f];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[f][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < NF) {
        const int f = threadIdx.x;
        atomicAdd(&out[(size_t)f * ntgt + ti], (double)((red[f][0] + red[f][1]) + (red[f][2] + red[f][3])));
    }
}

// Sum over the sources src[0, cnt) of one staged piece of a source leaf
// (lane group grp of ngr) for the lane's target: compensated FP32 (TwoSum
// hi + lo), since the per-atom terms are much larger than their neutral
// total.  The contraction adds each pair into a plain FP32 block sum that
// is folded into (hi, lo) every four pairs: the block sum's rounding is of
// the order of a single pair's, and the TwoSum cost is paid once per four
// pairs.  k0 is the sorted index of src[0].  CHECK: the piece may hold the
// target itself or one of its excluded partners.
template <int M, int F, int DAMP, bool CHECK>
__device__ __forceinline__ void p2p_leaf(const float4* src, int cnt, int k0, int grp, int ngr, int tgt, float xt,
                                         float yt, float zt, float dt, float ox, float oy, float oz, float oxl,
                                         float oyl, float ozl, const int32_t* __restrict__ excl, int exw, int64_t n,
                                         int ot, float* hi, float* lo) {
    constexpr int NF = nT(F), NM = nT(M), NV = rec_vec(NM);
    float blk[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) blk[f] = 0.0f;
    int nb = 0;
    for (int k = grp; k < cnt; k += ngr) {
        const float4* r = src + k * NV;
        const float4 a = r[0], b = r[1];
        if (CHECK) {
            if (k0 + k == tgt) continue;
            const int o = __float_as_int(b.w);
            bool skip = false;
            for (int e = 0; e < exw; ++e) skip |= (excl[(size_t)e * n + ot] == o);
            if (skip) continue;
        }
        float mc[4 * (NV - 2)];
#pragma unroll
        for (int v = 0; v < NV - 2; ++v) {
            const float4 w = r[2 + v];
            mc[4 * v] = w.x;
            mc[4 * v + 1] = w.y;
            mc[4 * v + 2] = w.z;
            mc[4 * v + 3] = w.w;
        }
        const float dx = ((xt - a.x) + ox) + (oxl - b.x);
        const float dy = ((yt - a.y) + oy) + (oyl - b.y);
        const float dz = ((zt - a.z) + oz) + (ozl - b.z);
        pair_field_f32acc<M, F>(dx, dy, dz, dt * a.w, DAMP, mc, blk);
        if (++nb == 4) {
            nb = 0;
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const float s = hi[f] + blk[f];
                const float bb = s - hi[f];
                lo[f] += (hi[f] - (s - bb)) + (blk[f] - bb);
                hi[f] = s;
                blk[f] = 0.0f;
            }
        }
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        const float s = hi[f] + blk[f];
        const float bb = s - hi[f];
        lo[f] += (hi[f] - (s - bb)) + (blk[f] - bb);
        hi[f] = s;
    }
}

// p2p_leaf on the packed records (k_gather_x2): blocks b = grp, grp + ngr,
// ... of the staged piece, each the lane's target against two sources in
// packed arithmetic.  Each half keeps its own compensated sum (H, L) over all
// pieces of the target chunk, fed from a plain block sum B folded every four
// blocks (four pairs per fold per half, as in the scalar loop).  The target
// position enters as xo = x_t + (c_A - c_B)_hi per piece and the low parts as
// oxl, so R = (xo - x_s) + (oxl - x_s,lo).  k0 is the sorted index of slot 0.
// CORR (a piece of a far leaf inside the damping range): only the damping
// correction (damped minus undamped kernel) of the pairs with (a r)^2 below
// xcut2, beyond which the damped kernel equals the undamped one to the
// requested accuracy; a block is skipped when no lane has such a pair.
template <int M, int F, int DAMP, bool CHECK, bool CORR = false>
__device__ __forceinline__ void p2p_leaf_x2(const float4* src, int nblk, int k0, int grp, int ngr, int tgt, f2 xo,
                                            f2 yo, f2 zo, f2 dt, f2 oxl, f2 oyl, f2 ozl,
                                            const int32_t* __restrict__ excl, int exw, int64_t n, int ot, f2* H,
                                            f2* L, float xcut2 = 0.0f, int* ncorr = nullptr) {
    constexpr int NF = nT(F), NM = nT(M), NV = rec_vec(NM), NE = 4 * (NV - 2);
    f2 B[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) B[f] = bc2(0.0f);
    int nb = 0;
    for (int b = grp; b < nblk; b += ngr) {
        const ulonglong2* r = reinterpret_cast<const ulonglong2*>(src + (size_t)b * 2 * NV);
        // element pairs: (x, y), (z, d), (x_lo, y_lo), (z_lo, index), multipoles
        const ulonglong2 v0 = r[0], v1 = r[1];
        if constexpr (CORR) {
            const f2 cx = xo - f2{v0.x}, cy = yo - f2{v0.y}, cz = zo - f2{v1.x};
            const f2 aa = dt * f2{v1.y};
            const f2 tt = (aa * aa) * fma2(cx, cx, fma2(cy, cy, cz * cz));
            float t0, t1;
            sp2(tt, t0, t1);
            if (!__any_sync(__activemask(), t0 < xcut2 || t1 < xcut2)) continue;
            *ncorr += (t0 < xcut2 ? 1 : 0) + (t1 < xcut2 ? 1 : 0);  // pairs whose correction is needed
        }
        const ulonglong2 v2 = r[2], v3 = r[3];
        f2 mc[NE];
#pragma unroll
        for (int v = 0; v < NE / 2; ++v) {
            const ulonglong2 w = r[4 + v];
            mc[2 * v].v = w.x;
            mc[2 * v + 1].v = w.y;
        }
        f2 dx = (xo - f2{v0.x}) + (oxl - f2{v2.x});
        const f2 dy = (yo - f2{v0.y}) + (oyl - f2{v2.y});
        const f2 dz = (zo - f2{v1.x}) + (ozl - f2{v3.x});
        const f2 a = dt * f2{v1.y};
        if (CHECK) {
            float o0, o1;
            sp2(f2{v3.y}, o0, o1);
            const int k = k0 + 2 * b;
            bool s0 = k == tgt, s1 = k + 1 == tgt;
            for (int e = 0; e < exw; ++e) {
                const int x = excl[(size_t)e * n + ot];
                s0 |= x == __float_as_int(o0);
                s1 |= x == __float_as_int(o1);
            }
            if (s0 || s1) {
                // a skipped half gets zero multipoles at a finite distance
                const f2 keep = mk2(s0 ? 0.0f : 1.0f, s1 ? 0.0f : 1.0f);
#pragma unroll
                for (int e = 0; e < NE; ++e) mc[e] = mc[e] * keep;
                float d0, d1;
                sp2(dx, d0, d1);
                dx = mk2(s0 ? 1000.0f : d0, s1 ? 1000.0f : d1);
            }
        }
        pair_field_x2<M, F, CORR>(dx, dy, dz, a, DAMP, mc, B);
        if (++nb == 4) {
            nb = 0;
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const f2 s = H[f] + B[f];
                const f2 bb = s - H[f];
                L[f] += (H[f] - (s - bb)) + (B[f] - bb);
                H[f] = s;
                B[f] = bc2(0.0f);
            }
        }
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        const f2 s = H[f] + B[f];
        const f2 bb = s - H[f];
        L[f] += (H[f] - (s - bb)) + (B[f] - bb);
        H[f] = s;
    }
}

// Source records are staged per warp in shared memory, double-buffered:
// while one piece (a source leaf, or `stage` / NV of its particles when it
// is larger) is evaluated, the next is copied with cp.async.  The staging
// size (float4s per buffer) is a launch parameter (dynamic shared memory).
constexpr int kStage = 320;  // default float4s per staging buffer

__device__ __forceinline__ void cp_async16(float4* smem, const float4* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// One warp per target leaf, its particles across the lanes (for leaves of
// fewer than 32 particles, groups of lanes split each source piece).
// Source leaves that hold neither the target nor an excluded partner of any
// of the warp's targets run without the exclusion test.
// DAMP is the damping kind as a template parameter: one specialised kernel
// per kind keeps the pair loop free of kind dispatch and its code small.
// Work: with `next` null, warp w takes leaf t.leaves[w]; otherwise the warps
// stay resident and take leaves order[0], order[1], ... (the target leaves
// by decreasing pair count) from the counter `next`, so the largest leaves
// start first and the last wave is made of the smallest.
// X2: sources from the packed records `srec` (k_gather_x2, padded leaf starts
// sstart) evaluated two at a time; otherwise srec = rec, sstart = t.start.
// With a damping-correction list (packed kernel, AMOEBA: t.corr_off) each
// target chunk walks it after its near list, passing over the entries whose
// leaf bound (lext) rules out a pair inside xcut2 for every lane, and counts
// the corrected pairs into corr_count.
template <int M, int F, int DAMP, bool X2>
__global__ void __launch_bounds__(256, 2) k_p2p_f32(const TreeDev t, const float4* __restrict__ rec,
                                                    const float4* __restrict__ srec,
                                                    const int32_t* __restrict__ sstart,
                                                    const float4* __restrict__ chi, const float4* __restrict__ clo,
                                                    const int32_t* __restrict__ excl, int exw, int64_t n,
                                                    double* __restrict__ fs, int stage,
                                                    const int32_t* __restrict__ order, unsigned* __restrict__ next,
                                                    float xcut2, unsigned long long* __restrict__ corr_count,
                                                    const float2* __restrict__ lext) {
    constexpr int NF = nT(F), NM = nT(M), NV = rec_vec(NM);
    // the damping-correction list is walked after the near list (packed
    // kernel, AMOEBA)
    constexpr bool kCorr = X2 && DAMP == DAMP_AMOEBA;
    extern __shared__ __align__(16) float4 sbuf_p2p[];
    const int cap = X2 ? (stage / NV) & ~1 : stage / NV;  // particles (slots) per staged piece
    const int lane = threadIdx.x & 31;
    float4* const bufs = sbuf_p2p + (size_t)(threadIdx.x >> 5) * 2 * stage;
    const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int ncorr = 0;  // corrected pairs evaluated by this lane
    for (int round = 0;; ++round) {
    int item;
    if (next) {
        unsigned v = 0;
        if (lane == 0) v = atomicAdd(next, 1u);
        item = (int)__shfl_sync(0xffffffffu, v, 0);
    } else {
        if (round > 0) break;
        item = w0;
    }
    if (item >= t.num_leaves) break;
    const int leaf = order ? order[item] : t.leaves[item];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    const int q0 = t.near_off[leaf], nn = t.near_off[leaf + 1] - q0;
    const int c0 = (kCorr && t.corr_off) ? t.corr_off[leaf] : 0;
    const int q1 = nn + ((kCorr && t.corr_off) ? t.corr_off[leaf + 1] - c0 : 0);
    // source leaf of list entry q: near entries [0, nn), then correction entries
    auto src_of = [&](int q) { return q < nn ? t.near_src[q0 + q] : t.corr_src[c0 + q - nn]; };
    const float4 ca = chi[leaf], cal = clo[leaf];
    // chunks of 32 targets, then the remaining rem < 32 in cs sub-chunks of
    // gs targets; a chunk of g targets runs ngr = 32 / g lane groups of g
    // lanes (any g), each taking every ngr-th block of each staged piece
    const int full = cnt >> 5, rem = cnt & 31;
    const int cs = rem ? kSubChunks[rem] : 0, gs = rem ? (rem + cs - 1) / cs : 1;
    for (int ci = 0; ci < full + cs; ++ci) {
        const int chunk = ci < full ? 32 * ci : 32 * full + (ci - full) * gs;
        const int g = ci < full ? 32 : gs;
        const int nt = min(g, cnt - chunk);
        const int ngr = 32 / g;
        const int tl = lane % g, grp = lane / g;
        const bool valid = tl < nt && grp < ngr;
        const int tgt = s0 + chunk + (valid ? tl : 0);
        const float4 ta = rec[(size_t)tgt * NV], tb = rec[(size_t)tgt * NV + 1];
        const int ot = __float_as_int(tb.w) - 1;
        // leaves of the target's excluded partners (-1: none)
        int exl[kExwRegs];
#pragma unroll
        for (int e = 0; e < kExwRegs; ++e) {
            int o = (e < exw) ? excl[(size_t)e * n + ot] : 0;
            exl[e] = o > 0 ? t.leaf_of[t.pos_of[o - 1]] : -1;
        }
        // per-target sums over all source leaves as double-float pairs (FP32
        // arithmetic; the FP64 pipe is the scarce one)
        float AH[NF], AL[NF];
        f2 XH[NF], XL[NF];  // packed kernel: one compensated sum per half
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            AH[f] = AL[f] = 0.0f;
            XH[f] = XL[f] = bc2(0.0f);
        }
        // current piece (q, off) of source leaf j = [js, js + jc); the first
        // one is staged before the loop
        // correction entries whose leaf cannot hold a pair that needs a
        // correction for any of this chunk's targets are passed over without
        // staging: for target t and leaf B, a r >= d_t dmin_B (|x_t - c_B| -
        // extent_B) (all lanes take part)
        auto next_entry = [&](int q) {
            if constexpr (kCorr) {
                const float txa = ta.x + ca.x, tya = ta.y + ca.y, tza = ta.z + ca.z;
                while (q < q1 && q >= nn) {
                    const int B = t.corr_src[c0 + q - nn];
                    bool need = false;
                    if (valid) {
                        const float4 cb = chi[B];
                        const float2 eb = lext[B];
                        const float dx = txa - cb.x, dy = tya - cb.y, dz = tza - cb.z;
                        const float rmin = fmaxf(sqrtf(dx * dx + dy * dy + dz * dz) - eb.x - 1e-2f, 0.0f);
                        const float xm = ta.w * eb.y * rmin;
                        need = xm * xm < xcut2;
                    }
                    if (__any_sync(0xffffffffu, need)) break;
                    ++q;
                }
            }
            return q;
        };
        int q = next_entry(0), off = 0, j = 0, js = 0, jc = 0;
        if (q < q1) {
            j = src_of(q);
            js = sstart[j];
            jc = t.count[j];
            if (X2) jc += jc & 1;  // padded to whole blocks
            const int pc = min(cap, jc);
            for (int i = lane; i < pc * NV; i += 32) cp_async16(&bufs[i], srec + (size_t)js * NV + i);
        }
        cp_async_commit();
        int slot = 0;
        while (q < q1) {
            // stage the next piece
            int nq = q, noff = off + cap, nj = j, njs = js, njc = jc;
            if (noff >= jc) {
                nq = next_entry(q + 1);
                noff = 0;
                if (nq < q1) {
                    nj = src_of(nq);
                    njs = sstart[nj];
                    njc = t.count[nj];
                    if (X2) njc += njc & 1;
                }
            }
            if (nq < q1) {
                const int npc = min(cap, njc - noff);
                const float4* gsrc = srec + (size_t)(njs + noff) * NV;
                float4* dst = bufs + (slot ^ 1) * stage;
                for (int i = lane; i < npc * NV; i += 32) cp_async16(&dst[i], gsrc + i);
            }
            cp_async_commit();
            cp_async_wait_prev();
            __syncwarp();
            if (valid) {
                // leaf-centre offset c_A - c_B as hi + lo; the low parts are
                // folded with the target's low parts
                const float4 cb = chi[j], cbl = clo[j];
                float ex, ey, ez;
                const float ox = two_diff(ca.x, cb.x, ex), oy = two_diff(ca.y, cb.y, ey), oz = two_diff(ca.z, cb.z, ez);
                const float oxl = (ex + (cal.x - cbl.x)) + tb.x, oyl = (ey + (cal.y - cbl.y)) + tb.y,
                            ozl = (ez + (cal.z - cbl.z)) + tb.z;
                bool need = (j == leaf) || exw > kExwRegs;
#pragma unroll
                for (int e = 0; e < kExwRegs; ++e) need |= (exl[e] == j);
                const int pc = min(cap, jc - off);
                const float4* cur = bufs + slot * stage;
                const int k0 = (X2 ? t.start[j] : js) + off;  // sorted index of the piece's first slot
                if constexpr (X2) {
                    const f2 xo = bc2(ta.x + ox), yo = bc2(ta.y + oy), zo = bc2(ta.z + oz), dt = bc2(ta.w);
                    const f2 oxl2 = bc2(oxl), oyl2 = bc2(oyl), ozl2 = bc2(ozl);
                    const bool anyneed = __any_sync(__activemask(), need);
                    if (kCorr && q >= nn) {
                        if constexpr (kCorr) {
                            if (anyneed)
                                p2p_leaf_x2<M, F, DAMP, true, true>(cur, pc >> 1, k0, grp, ngr, tgt, xo, yo, zo, dt,
                                                                    oxl2, oyl2, ozl2, excl, exw, n, ot, XH, XL, xcut2,
                                                                    &ncorr);
                            else
                                p2p_leaf_x2<M, F, DAMP, false, true>(cur, pc >> 1, k0, grp, ngr, tgt, xo, yo, zo, dt,
                                                                     oxl2, oyl2, ozl2, excl, exw, n, ot, XH, XL,
                                                                     xcut2, &ncorr);
                        }
                    } else if (anyneed)
                        p2p_leaf_x2<M, F, DAMP, true>(cur, pc >> 1, k0, grp, ngr, tgt, xo, yo, zo, dt, oxl2, oyl2,
                                                      ozl2, excl, exw, n, ot, XH, XL);
                    else
                        p2p_leaf_x2<M, F, DAMP, false>(cur, pc >> 1, k0, grp, ngr, tgt, xo, yo, zo, dt, oxl2, oyl2,
                                                       ozl2, excl, exw, n, ot, XH, XL);
                } else {
                    float hi[NF], lo[NF];
#pragma unroll
                    for (int f = 0; f < NF; ++f) hi[f] = lo[f] = 0.0f;
                    if (__any_sync(__activemask(), need))
                        p2p_leaf<M, F, DAMP, true>(cur, pc, k0, grp, ngr, tgt, ta.x, ta.y, ta.z, ta.w, ox, oy, oz,
                                                   oxl, oyl, ozl, excl, exw, n, ot, hi, lo);
                    else
                        p2p_leaf<M, F, DAMP, false>(cur, pc, k0, grp, ngr, tgt, ta.x, ta.y, ta.z, ta.w, ox, oy, oz,
                                                    oxl, oyl, ozl, excl, exw, n, ot, hi, lo);
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        // (AH, AL) += (hi, lo)
                        const float sum = AH[f] + hi[f];
                        const float bb = sum - AH[f];
                        const float err = (AH[f] - (sum - bb)) + (hi[f] - bb);
                        AH[f] = sum;
                        AL[f] += err + lo[f];
                    }
                }
            }
            __syncwarp();
            q = nq;
            off = noff;
            j = nj;
            js = njs;
            jc = njc;
            slot ^= 1;
        }
        cp_async_wait_all();
        __syncwarp();
        double acc[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            if constexpr (X2) {
                float h0, h1, l0, l1;
                sp2(XH[f], h0, h1);
                sp2(XL[f], l0, l1);
                acc[f] = ((double)h0 + (double)h1) + ((double)l0 + (double)l1);
            } else {
                acc[f] = (double)AH[f] + (double)AL[f];
            }
        }
        if ((g & (g - 1)) == 0) {
            for (int o = g; o < 32; o <<= 1) {
#pragma unroll
                for (int f = 0; f < NF; ++f) acc[f] += __shfl_xor_sync(0xffffffffu, acc[f], o);
            }
        } else {
            // group 0 adds groups 1 .. ngr - 1 (lanes tl + k g)
            double part[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) part[f] = acc[f];
            for (int k = 1; k < ngr; ++k) {
#pragma unroll
                for (int f = 0; f < NF; ++f) acc[f] += __shfl_sync(0xffffffffu, part[f], (tl + k * g) & 31);
            }
        }
        if (grp == 0 && valid) {
#pragma unroll
            for (int f = 0; f < NF; ++f) fs[(size_t)f * n + tgt] = acc[f];
        }
    }
    }
    if (kCorr && corr_count) {
        // every lane of the warp is here (leaves are taken per warp)
        const int sc = __reduce_add_sync(0xffffffffu, ncorr);
        if ((threadIdx.x & 31) == 0 && sc) atomicAdd(corr_count, (unsigned long long)sc);
    }
}

// Local field scale of each leaf for the learned selector's error budgets:
// the field (order-1 components, FP32, damped as the call) at up to
// kScaleSamples particles of the leaf from every particle of its smallest
// ancestor holding at least kScaleNeighbours particles (a subtree is one
// contiguous range of the sorted particles; at most kScaleWindow of them
// around the leaf), excluded partners and the
// particle itself skipped; the leaf's values are the mean and the minimum
// of log10 of the magnitudes found (-30 for a zero field), at scale[leaf]
// and scale[num_nodes + leaf].  The field at a particle is
// dominated by its nearest neighbours, which lie in that range except near
// the range's faces; the estimate sets how much absolute error each far pair
// may carry at the leaf.
constexpr int kScaleSamples = 4;
constexpr int kScaleNeighbours = 256;
constexpr int kScaleWindow = 1024;

template <int M>
__global__ void __launch_bounds__(128) k_leaf_field_scale(const TreeDev t, const float4* __restrict__ rec,
                                                          const float4* __restrict__ chi, int damp, int exw,
                                                          const int32_t* __restrict__ excl, int64_t n,
                                                          float* __restrict__ scale) {
    constexpr int NM = nT(M), NV = rec_vec(NM);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= t.num_leaves) return;
    const int leaf = t.leaves[w];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    int anc = leaf;
    while (t.count[anc] < kScaleNeighbours && t.parent[anc] >= 0) anc = t.parent[anc];
    // at most kScaleWindow particles of that range, centred on the leaf's
    // (Morton order keeps them near it)
    int a0 = t.start[anc], a1 = a0 + t.count[anc];
    if (a1 - a0 > kScaleWindow) {
        a0 = max(a0, min(s0 + cnt / 2 - kScaleWindow / 2, a1 - kScaleWindow));
        a1 = a0 + kScaleWindow;
    }
    const int ns = min(kScaleSamples, cnt);
    float lsum = 0.0f, lmin = 30.0f;
    for (int sidx = 0; sidx < ns; ++sidx) {
        const int k = s0 + (int)((int64_t)sidx * cnt / ns);
        const float4 ta = rec[(size_t)k * NV], tb = rec[(size_t)k * NV + 1];
        const float4 ca = chi[leaf];
        const float tx = ta.x + ca.x, ty = ta.y + ca.y, tz = ta.z + ca.z;
        const int ot = __float_as_int(tb.w) - 1;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int q = a0 + lane; q < a1; q += 32) {
            if (q == k) continue;
            const float4* r = rec + (size_t)q * NV;
            const float4 sa = r[0], sb = r[1];
            const int o = __float_as_int(sb.w);
            bool ex = false;
            for (int e = 0; e < exw; ++e) ex |= (excl[(size_t)e * n + ot] == o);
            if (ex) continue;
            const float4 cb = chi[t.leaf_of[q]];
            float mc[4 * (NV - 2)];
#pragma unroll
            for (int v = 0; v < NV - 2; ++v) {
                const float4 wv = r[2 + v];
                mc[4 * v] = wv.x;
                mc[4 * v + 1] = wv.y;
                mc[4 * v + 2] = wv.z;
                mc[4 * v + 3] = wv.w;
            }
            const float dx = tx - (sa.x + cb.x), dy = ty - (sa.y + cb.y), dz = tz - (sa.z + cb.z);
            if constexpr (M == 2) {
                // quadrupole sources: the dot-product contraction (the record's
                // pad slot holds the trace of the second moments)
                float g[4];
                radial_g<3, float>(damp, dx * dx + dy * dy + dz * dz, ta.w * sa.w, g);
                contract_q1<float>(dx, dy, dz, g, mc, mc[10], damp, acc);
            } else {
                pair_field<M, 1, float>(dx, dy, dz, ta.w * sa.w, damp, mc, acc);
            }
        }
#pragma unroll
        for (int c = 1; c < 4; ++c)
            for (int off = 16; off > 0; off >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], off);
        const float l = log10f(fmaxf(sqrtf(acc[1] * acc[1] + acc[2] * acc[2] + acc[3] * acc[3]), 1e-30f));
        lsum += l;
        lmin = fminf(lmin, l);
    }
    if (lane == 0) {
        scale[leaf] = ns > 0 ? lsum / (float)ns : -30.0f;
        scale[t.num_nodes + leaf] = ns > 0 ? lmin : -30.0f;
    }
}

// Pair work of each target leaf (its particles times the particles of its
// near list) for the work queue's order.
__global__ void k_leaf_cost(const TreeDev t, uint32_t* __restrict__ cost, int32_t* __restrict__ ids) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= t.num_leaves) return;
    const int leaf = t.leaves[w];
    uint32_t s = 0;
    for (int q = t.near_off[leaf] + lane; q < t.near_off[leaf + 1]; q += 32) s += (uint32_t)t.count[t.near_src[q]];
    if (t.corr_off) {
        // damping-correction pieces: mostly the cheap range test, about a
        // quarter of a near pair each
        uint32_t c = 0;
        for (int q = t.corr_off[leaf] + lane; q < t.corr_off[leaf + 1]; q += 32) c += (uint32_t)t.count[t.corr_src[q]];
        s += c / 4;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        const uint64_t c = (uint64_t)t.count[leaf] * s;
        cost[w] = c > 0xffffffffull ? 0xffffffffu : (uint32_t)c;
        ids[w] = leaf;
    }
}

template <int M, int F, bool X2>
void launch_p2p_kind(unsigned blocks, int threads, size_t smem, int stage, const int32_t* order, unsigned* next,
                     cudaStream_t st, const TreeDev& t, const float4* rec, const float4* srec, const int32_t* sstart,
                     const float4* chi, const float4* clo, const int32_t* excl, int exw, int64_t n, int damp,
                     double* fs, float xcut2, unsigned long long* corr_count, const float2* lext) {
    if constexpr (X2 && F > 1) {
        return;  // not instantiated: the packed kernel is used for field orders 0 and 1
    } else {
    switch (damp) {
        case DAMP_AMOEBA:
            k_p2p_f32<M, F, DAMP_AMOEBA, X2><<<blocks, threads, smem, st>>>(t, rec, srec, sstart, chi, clo, excl, exw,
                                                                              n, fs, stage, order, next, xcut2, corr_count, lext);
            break;
        case DAMP_THOLE:
            k_p2p_f32<M, F, DAMP_THOLE, X2><<<blocks, threads, smem, st>>>(t, rec, srec, sstart, chi, clo, excl, exw,
                                                                             n, fs, stage, order, next, xcut2, corr_count, lext);
            break;
        case DAMP_ERF:
            k_p2p_f32<M, F, DAMP_ERF, X2><<<blocks, threads, smem, st>>>(t, rec, srec, sstart, chi, clo, excl, exw, n,
                                                                           fs, stage, order, next, xcut2, corr_count, lext);
            break;
        default:
            k_p2p_f32<M, F, DAMP_NONE, X2><<<blocks, threads, smem, st>>>(t, rec, srec, sstart, chi, clo, excl, exw,
                                                                            n, fs, stage, order, next, xcut2, corr_count, lext);
            break;
    }
    }
}

template <int M, int F, bool X2>
const void* p2p_kernel(int damp) {
    if constexpr (X2 && F > 1) return nullptr;
    else
    return damp == DAMP_AMOEBA  ? (const void*)k_p2p_f32<M, F, DAMP_AMOEBA, X2>
           : damp == DAMP_THOLE ? (const void*)k_p2p_f32<M, F, DAMP_THOLE, X2>
           : damp == DAMP_ERF   ? (const void*)k_p2p_f32<M, F, DAMP_ERF, X2>
                                : (const void*)k_p2p_f32<M, F, DAMP_NONE, X2>;
}

template <int M, int F>
int set_p2p_smem(size_t smem) {
    const void* fns[8] = {p2p_kernel<M, F, false>(DAMP_NONE), p2p_kernel<M, F, false>(DAMP_AMOEBA),
                          p2p_kernel<M, F, false>(DAMP_THOLE), p2p_kernel<M, F, false>(DAMP_ERF),
                          p2p_kernel<M, F, true>(DAMP_NONE),  p2p_kernel<M, F, true>(DAMP_AMOEBA),
                          p2p_kernel<M, F, true>(DAMP_THOLE),  p2p_kernel<M, F, true>(DAMP_ERF)};
    for (const void* fn : fns)
        if (fn) FMM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return FMM_OK;
}

template <int M, int F>
int p2p_blocks_per_sm(int damp, bool x2, int threads, size_t smem) {
    int nb = 0;
    const void* fn = x2 ? p2p_kernel<M, F, true>(damp) : p2p_kernel<M, F, false>(damp);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return std::max(1, nb);
}

int num_sms_f32() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

}  // namespace

int prepare_f32_records(Workspace& ws, const Particles& P, const TreeDev& t, cudaStream_t st) {
    const int64_t n = P.n;
    const int nv = rec_vec(P.dim);
    FMM_TRY(ws.f32buf.ensure(sizeof(float4) * (size_t)n * nv));
    count_launches(1);
    k_gather_f32<<<grid_for(n, 256), 256, 0, st>>>(n, P.dim, t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                    ws.sz.as<double>(), ws.sd.as<double>(), ws.smc.as<double>(),
                                                    ws.f32buf.as<float4>());
    FMM_TRY(ws.f32node.ensure(sizeof(float4) * 2 * (size_t)t.num_nodes));
    float4* chi = ws.f32node.as<float4>();
    count_launches(1);
    k_node_centres_f32<<<grid_for(t.num_nodes, 256), 256, 0, st>>>(t.num_nodes, t, chi, chi + t.num_nodes);
    FMM_CUDA_TRY(cudaGetLastError());
    ws.f32node_ok = true;
    return FMM_OK;
}

int launch_leaf_extent(Workspace& ws, const Particles& P, const TreeDev& t, cudaStream_t st) {
    FMM_TRY(ws.leaf_ext.ensure(sizeof(float2) * (size_t)t.num_nodes));
    count_launches(1);
    k_leaf_extent<<<grid_for((int64_t)t.num_leaves * 32, 128), 128, 0, st>>>(rec_vec(P.dim), t, ws.f32buf.as<float4>(),
                                                                             ws.leaf_ext.as<float2>());
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_direct_scale_f32(Workspace& ws, const Particles& P, const TreeDev& t, int field_order, double* d_out,
                            cudaStream_t st, int64_t ntgt, const int64_t* d_targets) {
    const int m = dim_to_order(P.dim);
    const int nf = nT(field_order);
    FMM_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(double) * (size_t)nf * ntgt, st));
    int64_t ks = std::max<int64_t>(1, (16LL * 152 + ntgt - 1) / ntgt);
    ks = std::min<int64_t>(ks, std::max<int64_t>(1, P.n / 1024));
    const int64_t chunk = (P.n + ks - 1) / ks;
    const float4* chi = ws.f32node.as<float4>();
    dim3 grid((unsigned)ntgt, (unsigned)ks);
    FMM_MF_SWITCH(m, field_order,
                  (k_direct_scale<MM, FF><<<grid, 128, 0, st>>>(t, ws.f32buf.as<float4>(), chi, d_targets, ntgt, P.n,
                                                                 P.damp_type, P.exw, P.excl, chunk, d_out)));
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_leaf_field_scale(Workspace& ws, const Particles& P, const TreeDev& t, float* d_scale, cudaStream_t st) {
    const int m = dim_to_order(P.dim);
    const float4* rec = ws.f32buf.as<float4>();  // prepare_f32_records
    const float4* chi = ws.f32node.as<float4>();
    const unsigned blocks = grid_for((int64_t)t.num_leaves * 32, 128);
    switch (m) {
        case 0:
            k_leaf_field_scale<0><<<blocks, 128, 0, st>>>(t, rec, chi, P.damp_type, P.exw, P.excl, P.n, d_scale);
            break;
        case 1:
            k_leaf_field_scale<1><<<blocks, 128, 0, st>>>(t, rec, chi, P.damp_type, P.exw, P.excl, P.n, d_scale);
            break;
        case 2:
            k_leaf_field_scale<2><<<blocks, 128, 0, st>>>(t, rec, chi, P.damp_type, P.exw, P.excl, P.n, d_scale);
            break;
        default:
            return FMM_ENOTSUP;
    }
    count_launches(1);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

bool p2p_packed_enabled(const P2pShape& sh, int field_order, int damp) {
    const char* pe = std::getenv("FMM_GB300_P2P_PACKED");
    return sh.pack && !(pe && pe[0] == '0') && field_order <= 1 && damp != DAMP_ERF;
}

bool P2pShape::valid() const {
    return (threads == 64 || threads == 128 || threads == 256) && stage >= 64 && stage <= 1024 && stage % 16 == 0 &&
           (queue == 0 || queue == 1) && (pack == 0 || pack == 1);
}

int launch_p2p_f32(Workspace& ws, const Particles& P, const TreeDev& t, int field_order, cudaStream_t st) {
    const int m = dim_to_order(P.dim);
    const int64_t n = P.n;
    const int nf = nT(field_order);
    const float4* rec = ws.f32buf.as<float4>();  // prepare_f32_records
    const float4* chi = ws.f32node.as<float4>();
    const float4* clo = chi + t.num_nodes;
    FMM_TRY(ws.fsorted.ensure(sizeof(double) * (size_t)n * nf));
    const P2pShape sh = ws.p2p_shape.valid() ? ws.p2p_shape : P2pShape{};
    const size_t smem = sizeof(float4) * 2 * (size_t)sh.stage * (sh.threads / 32);
    if (rec_vec(P.dim) > sh.stage) return FMM_EINVAL;
    // packed kernel: sources two at a time from the padded, interleaved
    // records, for field orders 0 and 1 (at order 2 the packed registers do
    // not fit) and all kernels but erf (whose Boys series, at a r^2 < 6 for
    // much of an erf near field, runs per half: measured slower than the
    // one-source kernel); FMM_GB300_P2P_PACKED=0 selects the one-source kernel
    const bool x2 = p2p_packed_enabled(sh, field_order, P.damp_type) && t.num_leaves > 0 &&
                    n + (int64_t)t.num_leaves < (int64_t)INT32_MAX;
    // a damping-correction list is walked by the packed kernel only; the
    // pairs it corrects are counted in counter 9
    if (t.ncorr > 0 && !(x2 && P.damp_type == DAMP_AMOEBA)) return FMM_ENOTSUP;
    FMM_TRY(ws.counters.ensure(sizeof(unsigned long long) * 32));
    unsigned long long* corr_count = ws.counters.as<unsigned long long>() + 9;
    FMM_CUDA_TRY(cudaMemsetAsync(corr_count, 0, sizeof(unsigned long long), st));
    // leaf extents: computed with the lists (launch_leaf_extent)
    const float2* lext = t.ncorr > 0 ? ws.leaf_ext.as<float2>() : nullptr;
    if (x2) {
        const int nv = rec_vec(P.dim);
        const int L = t.num_leaves;
        FMM_TRY(ws.f32x2.ensure(sizeof(float4) * (size_t)(n + L + 1) * nv));
        if (!ws.reuse_structure) {
            // padded leaf starts (structure: kept for replays)
            FMM_TRY(ws.p2p_pad.ensure(sizeof(int32_t) * ((size_t)t.num_nodes + 2 * (size_t)L)));
            int32_t* ps = ws.p2p_pad.as<int32_t>();
            int32_t* odd = ps + t.num_nodes;
            int32_t* pre = odd + L;
            count_launches(1);
            k_leaf_odd<<<grid_for(L, 256), 256, 0, st>>>(t, odd);
            size_t tb = 0;
            cub::DeviceScan::ExclusiveSum(nullptr, tb, odd, pre, L, st);
            FMM_TRY(ws.cub_tmp.ensure(tb));
            FMM_CUDA_TRY(cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tb, odd, pre, L, st));
            count_launches(1);
            k_leaf_pstart<<<grid_for(L, 256), 256, 0, st>>>(t, pre, ps);
        }
        count_launches(1);
        k_gather_x2<<<grid_for(n, 256), 256, 0, st>>>(n, nv, P.dim == 10 && field_order == 1, t,
                                                       ws.p2p_pad.as<int32_t>(), rec,
                                                       reinterpret_cast<float*>(ws.f32x2.as<float4>()));
    }
    const int32_t* order = nullptr;
    unsigned* next = nullptr;
    unsigned blocks = grid_for((int64_t)t.num_leaves * 32, sh.threads);
    if (sh.queue && t.num_leaves > 0) {
        // target leaves by decreasing pair work (structure: kept for replays)
        FMM_TRY(ws.counters.ensure(sizeof(unsigned long long) * 32));
        next = reinterpret_cast<unsigned*>(ws.counters.as<unsigned long long>() + 11);
        if (!ws.reuse_structure) {
            const int L = t.num_leaves;
            FMM_TRY(ws.p2p_order.ensure(sizeof(int32_t) * 2 * (size_t)L + sizeof(uint32_t) * 2 * (size_t)L));
            int32_t* ids = ws.p2p_order.as<int32_t>() + L;
            uint32_t* cost = reinterpret_cast<uint32_t*>(ws.p2p_order.as<int32_t>() + 2 * (size_t)L);
            uint32_t* cost2 = cost + L;
            count_launches(1);
            k_leaf_cost<<<grid_for((int64_t)L * 32, 128), 128, 0, st>>>(t, cost, ids);
            size_t tb = 0;
            cub::DeviceRadixSort::SortPairsDescending(nullptr, tb, cost, cost2, ids, ws.p2p_order.as<int32_t>(), L, 0,
                                                      32, st);
            FMM_TRY(ws.cub_tmp.ensure(tb));
            FMM_CUDA_TRY(cub::DeviceRadixSort::SortPairsDescending(ws.cub_tmp.p, tb, cost, cost2, ids,
                                                                   ws.p2p_order.as<int32_t>(), L, 0, 32, st));
        }
        order = ws.p2p_order.as<int32_t>();
        FMM_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(unsigned), st));
        int bps = 1;
        FMM_MF_SWITCH(m, field_order, (bps = p2p_blocks_per_sm<MM, FF>(P.damp_type, x2, sh.threads, smem)));
        blocks = (unsigned)std::min<int64_t>(blocks, (int64_t)bps * num_sms_f32());
    }
    if (smem > 48 * 1024) {
        FMM_MF_SWITCH(m, field_order, FMM_TRY((set_p2p_smem<MM, FF>(smem))));
    }
    if (x2) {
        FMM_MF_SWITCH(m, field_order,
                      (launch_p2p_kind<MM, FF, true>(blocks, sh.threads, smem, sh.stage, order, next, st, t, rec,
                                                     ws.f32x2.as<float4>(), ws.p2p_pad.as<int32_t>(), chi, clo,
                                                     P.excl, P.exw, n, P.damp_type, ws.fsorted.as<double>(),
                                                     ws.corr_xcut2, corr_count, lext)));
    } else {
        FMM_MF_SWITCH(m, field_order,
                      (launch_p2p_kind<MM, FF, false>(blocks, sh.threads, smem, sh.stage, order, next, st, t, rec, rec,
                                                      t.start, chi, clo, P.excl, P.exw, n, P.damp_type,
                                                      ws.fsorted.as<double>(), 0.0f, nullptr, nullptr)));
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

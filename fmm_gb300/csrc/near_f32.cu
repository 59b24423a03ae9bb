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
#include <algorithm>

#include "dispatch.cuh"
#include "internal.h"
#include "pair.cuh"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

constexpr int kExwRegs = 8;  // exclusion entries held in registers per target

// Positions relative to the particle's leaf centre as double-float pairs
// (hi = rounded value, lo = rounded remainder): differences of positions in
// two leaves then lose nothing beyond the final FP32 rounding.
__global__ void k_gather_f32(int64_t n, int dim, const TreeDev t, const double* __restrict__ sx,
                             const double* __restrict__ sy, const double* __restrict__ sz,
                             const double* __restrict__ sd, const double* __restrict__ smc, float* __restrict__ fx,
                             float* __restrict__ fy, float* __restrict__ fz, float* __restrict__ fxl,
                             float* __restrict__ fyl, float* __restrict__ fzl, float* __restrict__ fd,
                             float* __restrict__ fmc, int32_t* __restrict__ forig) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int leaf = t.leaf_of[k];
    const double rx = sx[k] - t.cx[leaf], ry = sy[k] - t.cy[leaf], rz = sz[k] - t.cz[leaf];
    fx[k] = (float)rx;
    fy[k] = (float)ry;
    fz[k] = (float)rz;
    fxl[k] = (float)(rx - (double)fx[k]);
    fyl[k] = (float)(ry - (double)fy[k]);
    fzl[k] = (float)(rz - (double)fz[k]);
    fd[k] = (float)sd[k];
    for (int c = 0; c < dim; ++c) fmc[(size_t)c * n + k] = (float)smc[(size_t)c * n + k];
    forig[k] = (int32_t)t.perm[k] + 1;  // 1-based, as in the exclusion lists
}

template <int M, int F>
__global__ void __launch_bounds__(128) k_p2p_f32(const TreeDev t, const float* __restrict__ fx,
                                                 const float* __restrict__ fy, const float* __restrict__ fz,
                                                 const float* __restrict__ fxl, const float* __restrict__ fyl,
                                                 const float* __restrict__ fzl, const float* __restrict__ fd,
                                                 const float* __restrict__ fmc,
                                                 const int32_t* __restrict__ forig, const int32_t* __restrict__ excl,
                                                 int exw, int64_t n, int damp, double* __restrict__ fs) {
    constexpr int NF = nT(F), NM = nT(M);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= t.num_leaves) return;
    const int leaf = t.leaves[w];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    const int q0 = t.near_off[leaf], q1 = t.near_off[leaf + 1];
    const double cxa = t.cx[leaf], cya = t.cy[leaf], cza = t.cz[leaf];
    for (int chunk = 0; chunk < cnt; chunk += 32) {
        const int nt = min(32, cnt - chunk);
        int g = 1;
        while (g < nt) g <<= 1;
        const int ngr = 32 / g;
        const int tl = lane & (g - 1), grp = lane / g;
        const bool valid = tl < nt;
        const int tgt = s0 + chunk + (valid ? tl : 0);
        const float xt = fx[tgt], yt = fy[tgt], zt = fz[tgt], dt = fd[tgt];
        const float xtl = fxl[tgt], ytl = fyl[tgt], ztl = fzl[tgt];
        const int ot = forig[tgt] - 1;
        int ex[kExwRegs];
#pragma unroll
        for (int q = 0; q < kExwRegs; ++q) ex[q] = (q < exw) ? excl[(size_t)q * n + ot] : 0;
        double acc[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) acc[f] = 0.0;
        if (valid) {
            for (int q = q0; q < q1; ++q) {
                const int j = t.near_src[q];
                const int js = t.start[j], je = js + t.count[j];
                const double odx = cxa - t.cx[j], ody = cya - t.cy[j], odz = cza - t.cz[j];
                const float ox = (float)odx, oy = (float)ody, oz = (float)odz;
                // low parts of the offset folded with the target's low parts
                const float oxl = (float)(odx - (double)ox) + xtl, oyl = (float)(ody - (double)oy) + ytl,
                            ozl = (float)(odz - (double)oz) + ztl;
                // per source leaf: compensated FP32 sums (hi + lo, TwoSum), since
                // the per-atom terms are much larger than their (neutral) total
                float hi[NF], lo[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) hi[f] = lo[f] = 0.0f;
                for (int k = js + grp; k < je; k += ngr) {
                    if (k == tgt) continue;
                    const int o = forig[k];
                    bool skip = false;
#pragma unroll
                    for (int e = 0; e < kExwRegs; ++e) skip |= (ex[e] == o);
                    for (int e = kExwRegs; e < exw; ++e) skip |= (excl[(size_t)e * n + ot] == o);
                    if (skip) continue;
                    float mc[NM];
#pragma unroll
                    for (int s = 0; s < NM; ++s) mc[s] = fmc[(size_t)s * n + k];
                    const float dx = ((xt - fx[k]) + ox) + (oxl - fxl[k]);
                    const float dy = ((yt - fy[k]) + oy) + (oyl - fyl[k]);
                    const float dz = ((zt - fz[k]) + oz) + (ozl - fzl[k]);
                    float c[NF];
#pragma unroll
                    for (int f = 0; f < NF; ++f) c[f] = 0.0f;
                    pair_field_f32acc<M, F>(dx, dy, dz, dt * fd[k], damp, mc, c);
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        const float s = hi[f] + c[f];
                        const float bb = s - hi[f];
                        lo[f] += (hi[f] - (s - bb)) + (c[f] - bb);
                        hi[f] = s;
                    }
                }
#pragma unroll
                for (int f = 0; f < NF; ++f) acc[f] += (double)hi[f] + (double)lo[f];
            }
        }
        for (int off = g; off < 32; off <<= 1) {
#pragma unroll
            for (int f = 0; f < NF; ++f) acc[f] += __shfl_xor_sync(0xffffffffu, acc[f], off);
        }
        if (grp == 0 && valid) {
#pragma unroll
            for (int f = 0; f < NF; ++f) fs[(size_t)f * n + tgt] = acc[f];
        }
    }
}

}  // namespace

int launch_p2p_f32(Workspace& ws, const Particles& P, const TreeDev& t, int field_order, cudaStream_t st) {
    const int m = dim_to_order(P.dim);
    const int64_t n = P.n;
    const int nf = nT(field_order);
    FMM_TRY(ws.f32buf.ensure(sizeof(float) * (size_t)n * (7 + P.dim) + sizeof(int32_t) * n));
    float* fx = ws.f32buf.as<float>();
    float* fy = fx + n;
    float* fz = fy + n;
    float* fxl = fz + n;
    float* fyl = fxl + n;
    float* fzl = fyl + n;
    float* fd = fzl + n;
    float* fmc = fd + n;
    int32_t* forig = reinterpret_cast<int32_t*>(fmc + (size_t)n * P.dim);
    count_launches(1);
    k_gather_f32<<<grid_for(n, 256), 256, 0, st>>>(n, P.dim, t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                    ws.sz.as<double>(), ws.sd.as<double>(), ws.smc.as<double>(), fx,
                                                    fy, fz, fxl, fyl, fzl, fd, fmc, forig);
    FMM_TRY(ws.fsorted.ensure(sizeof(double) * (size_t)n * nf));
    const unsigned blocks = grid_for((int64_t)t.num_leaves * 32, 128);
    FMM_MF_SWITCH(m, field_order,
                  (k_p2p_f32<MM, FF><<<blocks, 128, 0, st>>>(t, fx, fy, fz, fxl, fyl, fzl, fd, fmc, forig, P.excl,
                                                              P.exw, n,
                                                              P.damp_type, ws.fsorted.as<double>())));
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

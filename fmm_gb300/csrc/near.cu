// Near field (P2P), direct sum and the exclusion corrections, FP64.
//
// Reference: particle_fields (src/fmm.F90:623-747) and particle_fields_direct
// (src/fmm.F90:749-824).  Both loop over target particles and call
// multipole_field on a vector of sources, moving excluded sources to
// R = (1e10, 1e10, 1e10).  Here the hot loops evaluate every source except the
// target itself, and a separate per-target pass fixes up the (few) excluded
// partners: it subtracts their contribution again and, in reference mode,
// adds the contribution at R = (1e10, 1e10, 1e10) that the reference keeps
// (a small potential term, src/fmm.F90:714-720).
#include <algorithm>

#include "internal.h"
#include "pair.cuh"
#include "dispatch.cuh"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

int num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

// Contraction coefficients c_s of the multipole components (order <= 3),
// folded at compile time (no FP64 division per element).
__constant__ double cSrcCoef[20] = {src_coef(0),  src_coef(1),  src_coef(2),  src_coef(3),  src_coef(4),
                                    src_coef(5),  src_coef(6),  src_coef(7),  src_coef(8),  src_coef(9),
                                    src_coef(10), src_coef(11), src_coef(12), src_coef(13), src_coef(14),
                                    src_coef(15), src_coef(16), src_coef(17), src_coef(18), src_coef(19)};

// Multipoles times the contraction coefficient c_s, original particle order.
__global__ void k_scale_mp(int64_t n, int dim, const double* __restrict__ mp, double* __restrict__ out) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    for (int c = 0; c < dim; ++c) out[(size_t)c * n + k] = cSrcCoef[c] * mp[(size_t)c * n + k];
}

// Particle data in key-sorted order (coordinates, damping, scaled multipoles).
__global__ void k_gather(int64_t n, int dim, const uint32_t* __restrict__ perm, const double* __restrict__ X,
                         const double* __restrict__ mp, const double* __restrict__ damp, double* __restrict__ sx,
                         double* __restrict__ sy, double* __restrict__ sz, double* __restrict__ sd,
                         double* __restrict__ smc) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t o = perm[k];
    sx[k] = X[o];
    sy[k] = X[n + o];
    sz[k] = X[2 * n + o];
    sd[k] = damp ? damp[o] : 0.0;
    for (int c = 0; c < dim; ++c) smc[(size_t)c * n + k] = cSrcCoef[c] * mp[(size_t)c * n + o];
}

// P2P: one warp per target leaf.  A leaf's targets are taken 32 at a time;
// when a chunk has g <= 16 targets (g rounded up to a power of two), the warp
// splits into 32/g groups that walk disjoint subsets of the sources, and the
// groups are summed with shuffles at the end, so few lanes idle.
// IMG: the lists are those of a periodic image (t.shift, t.central): sources
// sit at x_j + shift, the self pair counts unless the image is the central
// one, and the result is added to fs (src/fmm.F90:704-736).
template <int M, int F, bool IMG>
__global__ void __launch_bounds__(128) k_p2p_f64(const TreeDev t, const double* __restrict__ sx,
                                                 const double* __restrict__ sy, const double* __restrict__ sz,
                                                 const double* __restrict__ sd, const double* __restrict__ smc,
                                                 int64_t n, int damp, double* __restrict__ fs) {
    constexpr int NF = nT(F), NM = nT(M);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= t.num_leaves) return;
    const int leaf = t.leaves[w];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    const int q0 = t.near_off[leaf], q1 = t.near_off[leaf + 1];
    for (int chunk = 0; chunk < cnt; chunk += 32) {
        const int nt = min(32, cnt - chunk);
        int g = 1;
        while (g < nt) g <<= 1;
        const int ngr = 32 / g;
        const int tl = lane & (g - 1), grp = lane / g;
        const bool valid = tl < nt;
        const int tgt = s0 + chunk + (valid ? tl : 0);
        const double xt = sx[tgt], yt = sy[tgt], zt = sz[tgt], dt = sd[tgt];
        double acc[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) acc[f] = 0.0;
        if (valid) {
            for (int q = q0; q < q1; ++q) {
                const int j = t.near_src[q];
                const int js = t.start[j], je = js + t.count[j];
                for (int k = js + grp; k < je; k += ngr) {
                    if (k == tgt && (!IMG || t.central)) continue;
                    double mc[NM];
#pragma unroll
                    for (int s = 0; s < NM; ++s) mc[s] = smc[(size_t)s * n + k];
                    if (IMG)
                        pair_field<M, F, double>(xt - (sx[k] + t.shift[0]), yt - (sy[k] + t.shift[1]),
                                                 zt - (sz[k] + t.shift[2]), dt * sd[k], damp, mc, acc);
                    else
                        pair_field<M, F, double>(xt - sx[k], yt - sy[k], zt - sz[k], dt * sd[k], damp, mc, acc);
                }
            }
        }
        for (int off = g; off < 32; off <<= 1) {
#pragma unroll
            for (int f = 0; f < NF; ++f) acc[f] += __shfl_xor_sync(0xffffffffu, acc[f], off);
        }
        if (grp == 0 && valid) {
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                if (IMG)
                    fs[(size_t)f * n + tgt] += acc[f];
                else
                    fs[(size_t)f * n + tgt] = acc[f];
            }
        }
    }
}

// Direct sum: 128 targets per block, sources streamed through shared memory
// in tiles of 128; blockIdx.y splits the sources, partial sums per split.
template <int M, int F>
__global__ void __launch_bounds__(128) k_direct_f64(int64_t n, const int64_t* __restrict__ targets, int64_t ntgt,
                                                    const double* __restrict__ X, const double* __restrict__ mc,
                                                    const double* __restrict__ damp, int damp_type, int64_t chunk,
                                                    double* __restrict__ partial) {
    constexpr int NF = nT(F), NM = nT(M);
    constexpr int TILE = 128;
    __shared__ double shx[TILE], shy[TILE], shz[TILE], shd[TILE], shm[NM][TILE];
    const int64_t ti = blockIdx.x * (int64_t)TILE + threadIdx.x;
    const bool valid = ti < ntgt;
    const int64_t i = valid ? (targets ? targets[ti] : ti) : 0;
    const double xi = X[i], yi = X[n + i], zi = X[2 * n + i];
    const double di = damp ? damp[i] : 0.0;
    double acc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) acc[f] = 0.0;
    const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    for (int64_t jt = j0; jt < j1; jt += TILE) {
        const int64_t j = jt + threadIdx.x;
        if (j < j1) {
            shx[threadIdx.x] = X[j];
            shy[threadIdx.x] = X[n + j];
            shz[threadIdx.x] = X[2 * n + j];
            shd[threadIdx.x] = damp ? damp[j] : 0.0;
#pragma unroll
            for (int s = 0; s < NM; ++s) shm[s][threadIdx.x] = mc[(size_t)s * n + j];
        }
        __syncthreads();
        const int lim = (int)min((int64_t)TILE, j1 - jt);
        for (int k = 0; k < lim; ++k) {
            if (jt + k == i) continue;
            double m[NM];
#pragma unroll
            for (int s = 0; s < NM; ++s) m[s] = shm[s][k];
            pair_field<M, F, double>(xi - shx[k], yi - shy[k], zi - shz[k], di * shd[k], damp_type, m, acc);
        }
        __syncthreads();
    }
    if (valid) {
#pragma unroll
        for (int f = 0; f < NF; ++f) partial[((size_t)blockIdx.y * NF + f) * ntgt + ti] = acc[f];
    }
}

// Direct sum for a few targets: one block per (target, source split), the
// block's threads stride over the sources; block reduction of the partial
// field into partial[split][f][target].
template <int M, int F>
__global__ void __launch_bounds__(128) k_direct_few(int64_t n, const int64_t* __restrict__ targets, int64_t ntgt,
                                                    const double* __restrict__ X, const double* __restrict__ mc,
                                                    const double* __restrict__ damp, int damp_type, int64_t chunk,
                                                    double* __restrict__ partial) {
    constexpr int NF = nT(F), NM = nT(M);
    __shared__ double red[NF][4];
    const int64_t ti = blockIdx.x;
    const int64_t i = targets ? targets[ti] : ti;
    const double xi = X[i], yi = X[n + i], zi = X[2 * n + i];
    const double di = damp ? damp[i] : 0.0;
    double acc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) acc[f] = 0.0;
    const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
        if (j == i) continue;
        double m[NM];
#pragma unroll
        for (int s = 0; s < NM; ++s) m[s] = mc[(size_t)s * n + j];
        pair_field<M, F, double>(xi - X[j], yi - X[n + j], zi - X[2 * n + j], di * (damp ? damp[j] : 0.0), damp_type,
                                 m, acc);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        double v = acc[f];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[f][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < NF) {
        const int f = threadIdx.x;
        partial[((size_t)blockIdx.y * NF + f) * ntgt + ti] = (red[f][0] + red[f][1]) + (red[f][2] + red[f][3]);
    }
}

__global__ void k_direct_reduce(int64_t ntgt, int nf, int ks, const double* __restrict__ partial,
                                const int64_t* __restrict__ targets, int64_t ld, double* __restrict__ field) {
    const int64_t ti = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ti >= ntgt) return;
    const int64_t i = targets ? ti : ti;
    for (int f = 0; f < nf; ++f) {
        double s = 0.0;
        for (int k = 0; k < ks; ++k) s += partial[((size_t)k * nf + f) * ntgt + ti];
        field[(size_t)f * ld + i] = s;
    }
}

__device__ __forceinline__ bool is_near_leaf(const int32_t* near_off, const int32_t* near_src, int li, int lj) {
    int a = near_off[li], h = near_off[li + 1];
    while (a < h) {
        const int mid = (a + h) >> 1;
        if (near_src[mid] < lj)
            a = mid + 1;
        else
            h = mid;
    }
    return a < near_off[li + 1] && near_src[a] == lj;
}

// Exclusion fix-up, one thread per particle (original index i).  With a tree
// (FMM) the field is indexed by sorted position and "near" means the partner's
// leaf is in the near list of the target's leaf; without one (direct sum) every
// partner was evaluated by the hot loop.
template <int M, int F>
__global__ void k_excl_fix(int64_t n, int64_t ntgt, const int64_t* __restrict__ targets, const double* __restrict__ X,
                           const double* __restrict__ mc, int exw, const int32_t* __restrict__ excl,
                           const double* __restrict__ damp, int damp_type, int excl_mode,
                           const int32_t* __restrict__ pos_of, const int32_t* __restrict__ leaf_of,
                           const int32_t* __restrict__ near_off, const int32_t* __restrict__ near_src,
                           double* __restrict__ field, int64_t ld, int near_masked) {
    constexpr int NF = nT(F), NM = nT(M);
    const int64_t ti = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ti >= ntgt) return;
    const int64_t i = targets ? targets[ti] : ti;
    const bool fmm = pos_of != nullptr;
    const int64_t ki = fmm ? pos_of[i] : ti;
    const double xi = X[i], yi = X[n + i], zi = X[2 * n + i];
    const double di = damp ? damp[i] : 0.0;
    double add[NF], sub[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) add[f] = sub[f] = 0.0;
    bool self_listed = false;
    for (int w = 0; w < exw; ++w) {
        const int e = excl[(size_t)w * n + i];
        if (e == 0) continue;
        bool dup = false;
        for (int w2 = 0; w2 < w; ++w2)
            if (excl[(size_t)w2 * n + i] == e) dup = true;
        if (dup) continue;
        const int64_t j = e - 1;
        if (j == i) {
            self_listed = true;
            continue;
        }
        double m[NM];
#pragma unroll
        for (int s = 0; s < NM; ++s) m[s] = mc[(size_t)s * n + j];
        const double a = di * (damp ? damp[j] : 0.0);
        const bool near = fmm ? is_near_leaf(near_off, near_src, leaf_of[ki], leaf_of[pos_of[j]]) : true;
        if (near) {
            if (near_masked) continue;  // the near-field kernel already skipped this pair
            pair_field_cold<M, F, double>(xi - X[j], yi - X[n + j], zi - X[2 * n + j], a, damp_type, m, sub);
            if (excl_mode == 0) pair_field_cold<M, F, double>(1e10, 1e10, 1e10, a, damp_type, m, add);
        } else if (excl_mode == 1) {
            pair_field_cold<M, F, double>(xi - X[j], yi - X[n + j], zi - X[2 * n + j], 0.0, DAMP_NONE, m, sub);
        }
    }
    if (excl_mode == 0) {
        double m[NM];
#pragma unroll
        for (int s = 0; s < NM; ++s) m[s] = mc[(size_t)s * n + i];
        if (self_listed)
            pair_field_cold<M, F, double>(1e10, 1e10, 1e10, di * di, damp_type, m, add);
        else  // the reference evaluates the self pair at R = 0 (non-finite result)
            pair_field_cold<M, F, double>(0.0, 0.0, 0.0, di * di, damp_type, m, add);
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) field[(size_t)f * ld + ki] += add[f] - sub[f];
}

__global__ void k_scatter(int64_t n, int nf, const uint32_t* __restrict__ perm, const double* __restrict__ fs,
                          double* __restrict__ field) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t o = perm[k];
    for (int f = 0; f < nf; ++f) field[(size_t)f * n + o] = fs[(size_t)f * n + k];
}

}  // namespace

bool near_orders_supported(int m, int f) { return m >= 0 && m <= 3 && f >= 0 && f <= 3; }

int launch_direct_f64(Workspace& ws, const Particles& P, int field_order, const Modes& md, double* d_field,
                      cudaStream_t st, int64_t ntgt, const int64_t* d_targets, int split_cap) {
    const int m = dim_to_order(P.dim);
    if (!near_orders_supported(m, field_order)) return FMM_ENOTSUP;
    const int64_t n = P.n;
    if (!d_targets) ntgt = n;
    const int nf = nT(field_order);
    FMM_TRY(ws.dsmc.ensure(sizeof(double) * (size_t)n * P.dim));  // own buffer: may overlap the FMM phases
    double* mc = ws.dsmc.as<double>();
    count_launches(1);
    k_scale_mp<<<grid_for(n, 256), 256, 0, st>>>(n, P.dim, P.mp, mc);
    // few targets (sampled checks): a block per target and source split
    const bool few = ntgt <= 64;
    const int64_t tblocks = few ? ntgt : (ntgt + 127) / 128;
    int64_t ks = std::max<int64_t>(1, ((few ? 16LL : 8LL) * num_sms() + tblocks - 1) / tblocks);
    ks = std::min<int64_t>(ks, std::max<int64_t>(1, n / (few ? 1024 : 256)));
    ks = std::min<int64_t>(ks, 65535);
    if (split_cap > 0) ks = std::min<int64_t>(ks, split_cap);
    const int64_t chunk = (n + ks - 1) / ks;
    FMM_TRY(ws.partial.ensure(sizeof(double) * (size_t)ks * nf * ntgt));
    dim3 grid((unsigned)tblocks, (unsigned)ks);
    if (few) {
        FMM_MF_SWITCH_F64(m, field_order, (k_direct_few<MM, FF><<<grid, 128, 0, st>>>(n, d_targets, ntgt, P.x, mc, P.damp,
                                                                                   P.damp_type, chunk,
                                                                                   ws.partial.as<double>())));
    } else {
        FMM_MF_SWITCH_F64(m, field_order, (k_direct_f64<MM, FF><<<grid, 128, 0, st>>>(n, d_targets, ntgt, P.x, mc,
                                                                                   P.damp, P.damp_type, chunk,
                                                                                   ws.partial.as<double>())));
    }
    count_launches(1);
    k_direct_reduce<<<grid_for(ntgt, 256), 256, 0, st>>>(ntgt, nf, (int)ks, ws.partial.as<double>(), nullptr, ntgt,
                                                         d_field);
    if (P.exw > 0 || md.excl_mode == 0) {
        FMM_MF_SWITCH_F64(m, field_order,
                      (k_excl_fix<MM, FF><<<grid_for(ntgt, 128), 128, 0, st>>>(
                          n, ntgt, d_targets, P.x, mc, P.exw, P.excl, P.damp, P.damp_type, md.excl_mode, nullptr,
                          nullptr, nullptr, nullptr, d_field, ntgt, 0)));
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int gather_sorted(Workspace& ws, const Particles& P, const TreeDev& t, cudaStream_t st) {
    const int64_t n = P.n;
    FMM_TRY(ws.sx.ensure(sizeof(double) * n));
    FMM_TRY(ws.sy.ensure(sizeof(double) * n));
    FMM_TRY(ws.sz.ensure(sizeof(double) * n));
    FMM_TRY(ws.sd.ensure(sizeof(double) * n));
    FMM_TRY(ws.smc.ensure(sizeof(double) * (size_t)n * P.dim * 2));
    count_launches(1);
    k_gather<<<grid_for(n, 256), 256, 0, st>>>(n, P.dim, t.perm, P.x, P.mp, P.damp, ws.sx.as<double>(),
                                                ws.sy.as<double>(), ws.sz.as<double>(), ws.sd.as<double>(),
                                                ws.smc.as<double>());
    // original-order scaled multipoles for the exclusion pass
    count_launches(1);
    k_scale_mp<<<grid_for(n, 256), 256, 0, st>>>(n, P.dim, P.mp, ws.smc.as<double>() + (size_t)n * P.dim);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_p2p_f64(Workspace& ws, const Particles& P, const TreeDev& t, int field_order, const Modes& md,
                   cudaStream_t st, bool image) {
    (void)md;
    const int m = dim_to_order(P.dim);
    if (!near_orders_supported(m, field_order)) return FMM_ENOTSUP;
    const int64_t n = P.n;
    const int nf = nT(field_order);
    FMM_TRY(ws.fsorted.ensure(sizeof(double) * (size_t)n * nf));
    const unsigned blocks = grid_for((int64_t)t.num_leaves * 32, 128);
    if (image) {
        FMM_MF_SWITCH_F64(m, field_order,
                      (k_p2p_f64<MM, FF, true><<<blocks, 128, 0, st>>>(t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                                       ws.sz.as<double>(), ws.sd.as<double>(),
                                                                       ws.smc.as<double>(), n, P.damp_type,
                                                                       ws.fsorted.as<double>())));
    } else {
        FMM_MF_SWITCH_F64(m, field_order,
                      (k_p2p_f64<MM, FF, false><<<blocks, 128, 0, st>>>(t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                                        ws.sz.as<double>(), ws.sd.as<double>(),
                                                                        ws.smc.as<double>(), n, P.damp_type,
                                                                        ws.fsorted.as<double>())));
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_excl_correction(Workspace& ws, const Particles& P, const TreeDev* t, int field_order, const Modes& md,
                           double* d_field, cudaStream_t st) {
    const int m = dim_to_order(P.dim);
    const int64_t n = P.n;
    const double* mc_orig = ws.smc.as<double>() + (size_t)n * P.dim;
    FMM_MF_SWITCH_F64(m, field_order,
                  (k_excl_fix<MM, FF><<<grid_for(n, 128), 128, 0, st>>>(
                      n, n, nullptr, P.x, mc_orig, P.exw, P.excl, P.damp, P.damp_type, md.excl_mode, t->pos_of,
                      t->leaf_of, t->near_off, t->near_src, d_field, n,
                      (md.precision == 1 || md.precision == 2) ? 1 : 0)));
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int scatter_field(Workspace& ws, const TreeDev& t, int64_t n, int nf, double* d_field, cudaStream_t st) {
    count_launches(1);
    k_scatter<<<grid_for(n, 256), 256, 0, st>>>(n, nf, t.perm, ws.fsorted.as<double>(), d_field);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

// M2L in the harmonic (traceless) reduced basis, exact-coefficient modes.
//
// The reference's M2L (src/fmm.F90:826-882, multipole_field with pf = pm = p)
// evaluates, for every far pair, L_f += sum_{|s|<=p} c_s M_s T_{s+f} over all
// n_T(p) Cartesian components on both sides.  T_{k} = d^k (1/r) is harmonic,
// so on the source side d_z^2 can be replaced by -(d_x^2 + d_y^2): the weights
// w_s = c_s M_s of components with s_z >= 2 fold onto components with
// s_z <= 1 (exactly, order by order), leaving (p+1)^2 reduced moments w^_s.
// On the target side L is the derivative tensor of a harmonic potential, so
// only the (p+1)^2 components with f_z <= 1 are computed; the others follow
// from L_f = -L_{f-2z+2x} - L_{f-2z+2y}.  Both steps are exact identities of
// the undamped 1/r kernel, so the result equals the full Cartesian sum up to
// rounding, with (p+1)^4 instead of n_T(p)^2 multiply-adds per pair and only
// tensor components of z-index <= 2.
//
// One warp per target node; its sources in turn; the tensor (orders <= 2p,
// z-index <= 2) from the Hermite recursion in shared memory.  Lengths are
// scaled by the target half-width h (R' = R/h, w~_s = w^_s / h^|s|,
// L~_f = h^(|f|+1) L_f) so FP32 stays in range.  FP32 per-source results are
// added into FP64 accumulators every 8 sources.
#include <algorithm>

#include "internal.h"
#include "m2l_basis.cuh"
#include "pair.cuh"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }


// Fold w_s (full basis, in shared memory, length nT(p)) onto s_z <= 1.
__device__ void fold_moments(double* w, int p, int lane) {
    for (int tz = p - 2; tz >= 0; --tz) {
        // targets with z-index tz: components (tx, ty, tz), tx + ty <= p - tz
        const int m = p - tz;
        const int cnt = (m + 1) * (m + 2) / 2;
        for (int e = lane; e < cnt; e += 32) {
            int w2 = 0;
            while ((w2 + 1) * (w2 + 2) / 2 <= e) ++w2;  // tx + ty = w2
            const int ty = e - w2 * (w2 + 1) / 2;
            const int tx = w2 - ty;
            double v = 0.0;
            if (tx >= 2) v += w[pidx(tx - 2, ty, tz + 2)];
            if (ty >= 2) v += w[pidx(tx, ty - 2, tz + 2)];
            w[pidx(tx, ty, tz)] -= v;
        }
        __syncwarp();
    }
}

// Reduced source weights per node: w^_s = fold((-1)^(|s|+1) M'_s), s_z <= 1.
__global__ void k_reduce_moments(int M, int p, const double* __restrict__ mom, double* __restrict__ wred) {
    extern __shared__ double sm_fold[];
    const int nq = nT(p), nr = (p + 1) * (p + 1);
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* w = sm_fold + wib * nq;
    const int node = blockIdx.x * (blockDim.x >> 5) + wib;
    if (node >= M) return;
    for (int s = lane; s < nq; s += 32) {
        const double v = mom[(size_t)node * nq + s];
        w[s] = ((order_of(s) + 1) % 2) ? -v : v;
    }
    __syncwarp();
    fold_moments(w, p, lane);
    for (int q = lane; q < nr; q += 32) {
        const int c = qcomp(q);
        wred[(size_t)node * nr + q] = w[pidx(c & 0xff, (c >> 8) & 0xff, (c >> 16) & 0xff)];
    }
}

// Fills the f_z >= 2 components of each node's local expansion.
__global__ void k_complete_locals(int M, int p, double* __restrict__ loc) {
    const int node = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (node >= M) return;
    double* L = loc + (size_t)node * nT(p);
    for (int fz = 2; fz <= p; ++fz) {
        const int m = p - fz;
        const int cnt = (m + 1) * (m + 2) / 2;
        for (int e = lane; e < cnt; e += 32) {
            int w2 = 0;
            while ((w2 + 1) * (w2 + 2) / 2 <= e) ++w2;
            const int fy = e - w2 * (w2 + 1) / 2;
            const int fx = w2 - fy;
            L[pidx(fx, fy, fz)] = -L[pidx(fx + 2, fy, fz - 2)] - L[pidx(fx, fy + 2, fz - 2)];
        }
        __syncwarp();
    }
}

template <typename R>
struct Acc;
template <>
struct Acc<float> {
    static constexpr int kBlock = 8;  // sources summed in FP32 before an FP64 add
};
template <>
struct Acc<double> {
    static constexpr int kBlock = 1;
};

template <typename R, int RPL>
__global__ void __launch_bounds__(128) k_m2l_red(const TreeDev t, const double* __restrict__ wred,
                                                 double* __restrict__ loc, int p) {
    extern __shared__ double sm_raw[];
    const int N = 2 * p, nTr = rbase(N + 1), nr = (p + 1) * (p + 1), nq = nT(p);
    // block-shared tables
    int2* rule = reinterpret_cast<int2*>(sm_raw);
    size_t off = sizeof(int2) * nTr;
    off = (off + 15) & ~(size_t)15;
    R* wbase = reinterpret_cast<R*>(reinterpret_cast<char*>(sm_raw) + off);
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = 2 * nTr + nr + (N + 1) + 1;
    R* TA = wbase + wib * per_warp;
    R* TB = TA + nTr;
    R* ws = TB + nTr;
    R* gsh = ws + nr;
    // recursion rules of the restricted tensor entries
    for (int e = threadIdx.x; e < nTr; e += blockDim.x) rule[e] = restricted_rule(e);
    __syncthreads();
    const int i = blockIdx.x * (blockDim.x >> 5) + wib;
    if (i >= t.num_nodes) return;
    const double cxi = t.cx[i], cyi = t.cy[i], czi = t.cz[i];
    const double ih = 1.0 / t.r[i];
    const int q0 = t.far_off[i], q1 = t.far_off[i + 1];
    double acc[RPL];
    R part[RPL];
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
        acc[r] = 0.0;
        part[r] = (R)0;
    }
    // per-lane scale factors (1/h)^k for the reduced source entries it loads
    R sc[RPL];
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
        const int s = lane + 32 * r;
        double v = 1.0;
        if (s < nr) {
            const int k = (int)(qcomp(s) >> 24);
            for (int e = 0; e < k; ++e) v *= ih;
        }
        sc[r] = (R)v;
    }
    int fx_[RPL], fy_[RPL], fz_[RPL], fk_[RPL];
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
        const int c = (lane + 32 * r < nr) ? qcomp(lane + 32 * r) : 0;
        fx_[r] = c & 0xff;
        fy_[r] = (c >> 8) & 0xff;
        fz_[r] = (c >> 16) & 0xff;
        fk_[r] = c >> 24;
    }
    for (int q = q0; q < q1; ++q) {
        const int j = t.far_src[q];
        // per-pair expansion order (the far list stores it; at most p)
        const int pq = t.far_ord ? min((int)t.far_ord[q], p) : p;
        const int Nq = 2 * pq, nrq = (pq + 1) * (pq + 1);
        const R X = (R)((cxi - t.cx[j]) * ih), Y = (R)((cyi - t.cy[j]) * ih), Z = (R)((czi - t.cz[j]) * ih);
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
            const int s = lane + 32 * r;
            if (s < nrq) ws[s] = (R)wred[(size_t)j * nr + s] * sc[r];
        }
        const R r2 = X * X + Y * Y + Z * Z;
        const R rinv = Real<R>::rsqrt_(r2);
        const R rinv2 = rinv * rinv;
        if (lane <= Nq) {
            R v = rinv, c = (R)1;
            for (int jj = 1; jj <= lane; ++jj) {
                v *= rinv2;
                c *= -(R)(2 * jj - 1);
            }
            gsh[lane] = c * v;
        }
        __syncwarp();
        R* A = TA;
        R* B = TB;
        if (lane == 0) A[0] = gsh[Nq];
        __syncwarp();
        for (int lev = Nq - 1; lev >= 0; --lev) {
            const int lim = rbase(Nq - lev + 1);
            for (int e = lane; e < lim; e += 32) {
                R v;
                if (e == 0) {
                    v = gsh[lev];
                } else {
                    const int2 ru = rule[e];
                    const int dir = ru.x >> 16, cnt = ru.y >> 16;
                    const R crd = dir == 0 ? X : (dir == 1 ? Y : Z);
                    v = crd * A[ru.x & 0xffff];
                    if (cnt > 0) v += (R)cnt * A[ru.y & 0xffff];
                }
                B[e] = v;
            }
            __syncwarp();
            R* tmp = A;
            A = B;
            B = tmp;
        }
        // contraction over the reduced bases: sources by (order k, z-block sz,
        // y index); for a fixed output the tensor index then runs
        // contiguously along y, and each source weight is loaded once for all
        // of the lane's outputs
        {
            R a[RPL];
#pragma unroll
            for (int r = 0; r < RPL; ++r) a[r] = (R)0;
            for (int k = 0; k <= pq; ++k) {
#pragma unroll
                for (int sz = 0; sz <= 1; ++sz) {
                    const int len = k + 1 - sz;
                    if (len <= 0) continue;
                    const int soff = k * k + (sz == 0 ? 0 : k + 1);
                    int base[RPL];
#pragma unroll
                    for (int r = 0; r < RPL; ++r) {
                        const int n = k + fk_[r], v = sz + fz_[r];
                        base[r] = rbase(n) + (v == 0 ? 0 : (v == 1 ? n + 1 : 2 * n + 1)) + fy_[r];
                    }
                    for (int sy = 0; sy < len; ++sy) {
                        const R w = ws[soff + sy];
#pragma unroll
                        for (int r = 0; r < RPL; ++r)
                            if (lane + 32 * r < nrq) a[r] += w * A[base[r] + sy];
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < RPL; ++r) part[r] += a[r];
        }
        if (Acc<R>::kBlock == 1 || ((q - q0) % Acc<R>::kBlock) == Acc<R>::kBlock - 1) {
#pragma unroll
            for (int r = 0; r < RPL; ++r) {
                acc[r] += (double)part[r];
                part[r] = (R)0;
            }
        }
        __syncwarp();
    }
    double* L = loc + (size_t)i * nq;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
        const int f = lane + 32 * r;
        if (f < nr) {
            const int c = qcomp(f);
            const int k = c >> 24;
            double s = ih;
            for (int e = 0; e < k; ++e) s *= ih;
            L[pidx(c & 0xff, (c >> 8) & 0xff, (c >> 16) & 0xff)] = (acc[r] + (double)part[r]) * s;
        }
    }
}

int set_smem(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) FMM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return FMM_OK;
}

template <typename R, int RPL>
int launch_red_rpl(Workspace& ws, const TreeDev& t, int p, cudaStream_t st) {
    const int N = 2 * p, nTr = rbase(N + 1), nr = (p + 1) * (p + 1);
    size_t tab = sizeof(int2) * nTr;
    tab = (tab + 15) & ~(size_t)15;
    const size_t per_warp = sizeof(R) * (2 * nTr + nr + (N + 1) + 1);
    int wpb = 4;
    while (wpb > 1 && tab + wpb * per_warp > 160 * 1024) wpb /= 2;
    const size_t sm = tab + wpb * per_warp;
    FMM_TRY(set_smem((const void*)k_m2l_red<R, RPL>, sm));
    count_launches(1);
    k_m2l_red<R, RPL><<<grid_for(t.num_nodes, wpb), 32 * wpb, sm, st>>>(t, ws.wred.as<double>(), ws.loc.as<double>(),
                                                                        p);
    return FMM_OK;
}

// Outputs per lane: ceil((p+1)^2 / 32).
template <typename R>
int launch_red(Workspace& ws, const TreeDev& t, int p, cudaStream_t st) {
    const int rpl = ((p + 1) * (p + 1) + 31) / 32;
    if (rpl <= 1) return launch_red_rpl<R, 1>(ws, t, p, st);
    if (rpl <= 2) return launch_red_rpl<R, 2>(ws, t, p, st);
    if (rpl <= 3) return launch_red_rpl<R, 3>(ws, t, p, st);
    if (rpl <= 4) return launch_red_rpl<R, 4>(ws, t, p, st);
    return launch_red_rpl<R, 6>(ws, t, p, st);
}

}  // namespace

// Reduced source weights of every node at order p (into ws.wred).
int launch_reduce_moments(Workspace& ws, const TreeDev& t, int p, cudaStream_t st) {
    const int M = t.num_nodes, nq = nT(p), nr = (p + 1) * (p + 1);
    FMM_TRY(ws.wred.ensure(sizeof(double) * (size_t)M * nr));
    const int wpb = 4;
    const size_t sm = sizeof(double) * wpb * nq;
    FMM_TRY(set_smem((const void*)k_reduce_moments, sm));
    count_launches(1);
    k_reduce_moments<<<grid_for(M, wpb), 32 * wpb, sm, st>>>(M, p, ws.mom.as<double>(), ws.wred.as<double>());
    FMM_CUDA_TRY(cudaGetLastError());
    ws.wred_p = p;
    return FMM_OK;
}

// Exact-mode M2L: reduced moments, reduced M2L (FP32 or FP64), completion of
// the local expansions.
int launch_m2l_reduced(Workspace& ws, const TreeDev& t, int p, bool fp32, cudaStream_t st) {
    const int M = t.num_nodes, nq = nT(p), nr = (p + 1) * (p + 1);
    FMM_TRY(ws.loc.ensure(sizeof(double) * (size_t)M * nq));
    FMM_TRY(ws.wred.ensure(sizeof(double) * (size_t)M * nr));
    if (ws.wred_p != p) {  // not yet reduced from this call's moments
        const int wpb = 4;
        const size_t sm = sizeof(double) * wpb * nq;
        FMM_TRY(set_smem((const void*)k_reduce_moments, sm));
        count_launches(1);
        k_reduce_moments<<<grid_for(M, wpb), 32 * wpb, sm, st>>>(M, p, ws.mom.as<double>(), ws.wred.as<double>());
    }
    // (replays keep the choice between grouped products and the per-pair
    // kernel made when the structure was built)
    const int gst = (ws.reuse_structure && ws.m2l_pairwise) ? FMM_ENOTSUP : launch_m2l_grouped(ws, t, p, fp32, st);
    if (gst == FMM_ENOTSUP) {
        // per-pair kernel (FP64 operator too large for shared memory, or
        // displacement groups of a few pairs); in FP32 only up to order 8:
        // its tensors come from an FP32 recursion, which at higher orders
        // falls short of the mixed path's accuracy
        if (fp32 && p <= 8)
            FMM_TRY(launch_red<float>(ws, t, p, st));
        else
            FMM_TRY(launch_red<double>(ws, t, p, st));
    } else {
        FMM_TRY(gst);
    }
    count_launches(1);
    k_complete_locals<<<grid_for(M, 4), 128, 0, st>>>(M, p, ws.loc.as<double>());
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

// Multipole and local expansions, FP64: P2M, M2M, M2L, L2L, L2P.
//
// Cell multipoles are kept scaled, M'_t = M_t / t! (t! = tx! ty! tz!), where
// M_t are the reference's raw Cartesian moments sum q (r - c)^t.  Then every
// translation is a plain convolution with d^u / u!:
//   P2M  M'_t(leaf)   = sum_i sum_{s<=t} (d_i^(t-s)/(t-s)!) M'_s(i)   (src/fmm.F90:437-472)
//   M2M  M'_t(parent) = sum_c sum_{u<=t} (d_c^u/u!) M'_{t-u}(c)       (src/fmm.F90:387-435;
//        the reference shifts each leaf straight into every ancestor, which is
//        the same sum since the shifts compose exactly; here level by level)
//   M2L  L_f(i)      += sum_s (-1)^(|s|+1) M'_s(j) T_{s+f}(c_i - c_j)  (src/fmm.F90:826-882)
//   L2L  L_t(child)  += sum_u L_{t+u}(parent) d^u/u!                   (src/fmm.F90:981-1044)
//   L2P  F_t(i)      += sum_u L_{t+u}(leaf) d_i^u/u!, |t| <= f         (src/fmm.F90:1046-1132)
// Expansions are node-major: node k's coefficients are contiguous.
// All kernels use one warp per node; orders are runtime values up to 12.
#include <algorithm>
#include <vector>

#include "internal.h"
#include "pair.cuh"

namespace fmm {

namespace {

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

constexpr int kMaxNPL = (nT(kMaxP) + 31) / 32;  // per-lane accumulators

__device__ __forceinline__ int pack_comp(int q) { return comp_x(q) | (comp_y(q) << 8) | (comp_z(q) << 16); }
__device__ __forceinline__ int cx_(int c) { return c & 0xff; }
__device__ __forceinline__ int cy_(int c) { return (c >> 8) & 0xff; }
__device__ __forceinline__ int cz_(int c) { return (c >> 16) & 0xff; }

__device__ __forceinline__ void fill_comp(int* sh, int nq) {
    for (int q = threadIdx.x; q < nq; q += blockDim.x) sh[q] = pack_comp(q);
}

// e[a] = d^a / a!, a = 0..p
__device__ __forceinline__ void scaled_powers(double d, int p, double* e) {
    e[0] = 1.0;
    for (int a = 1; a <= p; ++a) e[a] = e[a - 1] * d / (double)a;
}

// dp[u] = dx^ux dy^uy dz^uz / u! for |u| <= p, computed by one warp.
__device__ __forceinline__ void warp_dpow(int lane, double dx, double dy, double dz, int p, const int* comp,
                                          double* e3, double* dp) {
    if (lane < 3) scaled_powers(lane == 0 ? dx : (lane == 1 ? dy : dz), p, e3 + lane * (kMaxP + 1));
    __syncwarp();
    for (int u = lane; u < nT(p); u += 32) {
        const int c = comp[u];
        dp[u] = e3[cx_(c)] * e3[(kMaxP + 1) + cy_(c)] * e3[2 * (kMaxP + 1) + cz_(c)];
    }
    __syncwarp();
}

// ---------------------------------------------------------------- P2M
__global__ void k_p2m(const TreeDev t, const double* __restrict__ sx, const double* __restrict__ sy,
                      const double* __restrict__ sz, const double* __restrict__ smc, int64_t n, int m, int p,
                      double* __restrict__ mom) {
    extern __shared__ double smem[];
    const int nq = nT(p);
    int* comp = reinterpret_cast<int*>(smem);
    double* base = smem + (nq + 1) / 2 + 1;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = nq + 3 * (kMaxP + 1) + 32;
    double* dp = base + wib * per_warp;
    double* e3 = dp + nq;
    double* ms = e3 + 3 * (kMaxP + 1);
    fill_comp(comp, nq);
    __syncthreads();
    const int w = blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= t.num_leaves) return;
    const int leaf = t.leaves[w];
    const double cx = t.cx[leaf], cy = t.cy[leaf], cz = t.cz[leaf];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    const int nm = nT(m);
    double acc[kMaxNPL];
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) acc[r] = 0.0;
    for (int k = s0; k < s0 + cnt; ++k) {
        if (lane < nm) {
            const double c = smc[(size_t)lane * n + k];
            ms[lane] = ((order_of(lane) + 1) % 2) ? -c : c;  // back to M_s / s!
        }
        warp_dpow(lane, sx[k] - cx, sy[k] - cy, sz[k] - cz, p, comp, e3, dp);
#pragma unroll
        for (int r = 0; r < kMaxNPL; ++r) {
            const int tq = lane + 32 * r;
            if (tq < nq) {
                const int ct = comp[tq];
                double a = 0.0;
                for (int s = 0; s < nm; ++s) {
                    const int cs = comp[s];
                    const int ux = cx_(ct) - cx_(cs), uy = cy_(ct) - cy_(cs), uz = cz_(ct) - cz_(cs);
                    if (ux < 0 || uy < 0 || uz < 0) continue;
                    a += dp[pidx(ux, uy, uz)] * ms[s];
                }
                acc[r] += a;
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) {
        const int tq = lane + 32 * r;
        if (tq < nq) mom[(size_t)leaf * nq + tq] = acc[r];
    }
}

// ---------------------------------------------------------------- M2M
__global__ void k_m2m(const TreeDev t, const int32_t* __restrict__ nodes, int cnt, int p, double* __restrict__ mom) {
    extern __shared__ double smem[];
    const int nq = nT(p);
    int* comp = reinterpret_cast<int*>(smem);
    double* base = smem + (nq + 1) / 2 + 1;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = 2 * nq + 3 * (kMaxP + 1);
    double* dp = base + wib * per_warp;
    double* mc = dp + nq;
    double* e3 = mc + nq;
    fill_comp(comp, nq);
    __syncthreads();
    const int w = blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= cnt) return;
    const int node = nodes[w];
    if (t.is_leaf[node]) return;
    const double px = t.cx[node], py = t.cy[node], pz = t.cz[node];
    double acc[kMaxNPL];
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) acc[r] = 0.0;
    for (int o = 0; o < 8; ++o) {
        const int c = t.child[8 * node + o];
        if (c < 0) continue;
        for (int q = lane; q < nq; q += 32) mc[q] = mom[(size_t)c * nq + q];
        warp_dpow(lane, t.cx[c] - px, t.cy[c] - py, t.cz[c] - pz, p, comp, e3, dp);
#pragma unroll
        for (int r = 0; r < kMaxNPL; ++r) {
            const int tq = lane + 32 * r;
            if (tq < nq) {
                const int ct = comp[tq];
                const int tx = cx_(ct), ty = cy_(ct), tz = cz_(ct);
                double a = 0.0;
                for (int ux = 0; ux <= tx; ++ux)
                    for (int uy = 0; uy <= ty; ++uy)
                        for (int uz = 0; uz <= tz; ++uz) a += dp[pidx(ux, uy, uz)] * mc[pidx(tx - ux, ty - uy, tz - uz)];
                acc[r] += a;
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) {
        const int tq = lane + 32 * r;
        if (tq < nq) mom[(size_t)node * nq + tq] = acc[r];
    }
}

// ---------------------------------------------------------------- M2L
// One warp per target node; sources of its far list in turn.  The tensor of
// orders <= 2p is built in shared memory, either by the Hermite recursion
// (exact) or by the reference's closed form with its Cnij table (ref mode,
// terms prepared on the host, evaluated in the reference's operation order).
__device__ __forceinline__ double ipow_rn(double x, int m) {
    unsigned nn = (unsigned)m;
    double y = (nn % 2) ? x : 1.0;
    while (nn >>= 1) {
        x = __dmul_rn(x, x);
        if (nn % 2) y = __dmul_rn(y, x);
    }
    return y;
}

__global__ void k_m2l_f64(const TreeDev t, const double* __restrict__ mom, double* __restrict__ loc, int p, int ref,
                          const int32_t* __restrict__ term_off, const uchar4* __restrict__ term_abc,
                          const double* __restrict__ term_c) {
    extern __shared__ double smem[];
    const int nq = nT(p), N = 2 * p, nqT = nT(N);
    int* comp = reinterpret_cast<int*>(smem);
    double* base = smem + (nqT + 1) / 2 + 1;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = 2 * nqT + nq + 5 * (N + 1);
    double* TA = base + wib * per_warp;
    double* TB = TA + nqT;
    double* ms = TB + nqT;
    double* gsh = ms + nq;     // g_j, or x powers in ref mode
    double* yp = gsh + (N + 1);
    double* zp = yp + (N + 1);
    double* ir = zp + (N + 1);
    fill_comp(comp, nqT);
    __syncthreads();
    const int i = blockIdx.x * (blockDim.x >> 5) + wib;
    if (i >= t.num_nodes) return;
    const double cxi = t.cx[i], cyi = t.cy[i], czi = t.cz[i];
    const int q0 = t.far_off[i], q1 = t.far_off[i + 1];
    int fcomp[kMaxNPL];
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) fcomp[r] = (lane + 32 * r < nq) ? comp[lane + 32 * r] : 0;
    double acc[kMaxNPL];
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) acc[r] = 0.0;
    for (int q = q0; q < q1; ++q) {
        const int j = t.far_src[q];
        const double X = __dsub_rn(cxi, __dadd_rn(t.cx[j], 0.0));
        const double Y = __dsub_rn(cyi, __dadd_rn(t.cy[j], 0.0));
        const double Z = __dsub_rn(czi, __dadd_rn(t.cz[j], 0.0));
        for (int s = lane; s < nq; s += 32) {
            const double v = mom[(size_t)j * nq + s];
            ms[s] = ((order_of(s) + 1) % 2) ? -v : v;  // (-1)^(|s|+1) M'_s
        }
        double* T;
        if (ref) {
            const double R = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(X, X), __dmul_rn(Y, Y)), __dmul_rn(Z, Z)));
            if (lane < 3) {
                const double v = lane == 0 ? X : (lane == 1 ? Y : Z);
                double* pw = lane == 0 ? gsh : (lane == 1 ? yp : zp);
                const double u = __ddiv_rn(v, R);
                pw[0] = 1.0;
                for (int a = 1; a <= N; ++a) pw[a] = __dmul_rn(pw[a - 1], u);
            }
            for (int k = lane; k <= N; k += 32) ir[k] = __ddiv_rn(1.0, ipow_rn(R, k + 1));
            __syncwarp();
            for (int c = lane; c < nqT; c += 32) {
                double a = 0.0;
                for (int tt = term_off[c]; tt < term_off[c + 1]; ++tt) {
                    const uchar4 e = term_abc[tt];
                    const double Cx = __dmul_rn(term_c[3 * tt], gsh[e.x]);
                    const double Cy = __dmul_rn(__dmul_rn(Cx, term_c[3 * tt + 1]), yp[e.y]);
                    a = __dadd_rn(a, __dmul_rn(__dmul_rn(Cy, term_c[3 * tt + 2]), zp[e.z]));
                }
                TA[c] = __dmul_rn(a, ir[order_of(c)]);
            }
            __syncwarp();
            T = TA;
        } else {
            const double r2 = X * X + Y * Y + Z * Z;
            const double rinv = rsqrt(r2);
            const double rinv2 = rinv * rinv;
            if (lane <= N) {
                // g_j = (-1)^j (2j-1)!! r^-(2j+1)
                double v = rinv, c = 1.0;
                for (int jj = 1; jj <= lane; ++jj) {
                    v *= rinv2;
                    c *= -(double)(2 * jj - 1);
                }
                gsh[lane] = c * v;
            }
            __syncwarp();
            // level N holds only g_N; descend to level 0
            double* A = TA;
            double* B = TB;
            if (lane == 0) A[0] = gsh[N];
            __syncwarp();
            for (int lev = N - 1; lev >= 0; --lev) {
                const int lim = nT(N - lev);
                for (int c = lane; c < lim; c += 32) {
                    double v;
                    if (c == 0) {
                        v = gsh[lev];
                    } else {
                        const int cc = comp[c];
                        const int tx = cx_(cc), ty = cy_(cc), tz = cz_(cc);
                        if (tx > 0) {
                            v = X * A[pidx(tx - 1, ty, tz)];
                            if (tx > 1) v += (double)(tx - 1) * A[pidx(tx - 2, ty, tz)];
                        } else if (ty > 0) {
                            v = Y * A[pidx(tx, ty - 1, tz)];
                            if (ty > 1) v += (double)(ty - 1) * A[pidx(tx, ty - 2, tz)];
                        } else {
                            v = Z * A[pidx(tx, ty, tz - 1)];
                            if (tz > 1) v += (double)(tz - 1) * A[pidx(tx, ty, tz - 2)];
                        }
                    }
                    B[c] = v;
                }
                __syncwarp();
                double* tmp = A;
                A = B;
                B = tmp;
            }
            T = A;
        }
        // contraction: L_f += sum_s ms_s T_{s+f}
#pragma unroll
        for (int r = 0; r < kMaxNPL; ++r) {
            if (lane + 32 * r < nq) {
                const int fx = cx_(fcomp[r]), fy = cy_(fcomp[r]), fz = cz_(fcomp[r]);
                double a = 0.0;
                for (int s = 0; s < nq; ++s) {
                    const int cs = comp[s];
                    a += ms[s] * T[pidx(cx_(cs) + fx, cy_(cs) + fy, cz_(cs) + fz)];
                }
                acc[r] += a;
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) {
        const int fq = lane + 32 * r;
        if (fq < nq) loc[(size_t)i * nq + fq] = acc[r];
    }
}


// ---------------------------------------------------------------- L2L
__global__ void k_l2l(const TreeDev t, const int32_t* __restrict__ nodes, int cnt, int p, double* __restrict__ loc) {
    extern __shared__ double smem[];
    const int nq = nT(p);
    int* comp = reinterpret_cast<int*>(smem);
    double* base = smem + (nq + 1) / 2 + 1;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = 2 * nq + 3 * (kMaxP + 1);
    double* dp = base + wib * per_warp;
    double* lp = dp + nq;
    double* e3 = lp + nq;
    fill_comp(comp, nq);
    __syncthreads();
    const int w = blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= cnt) return;
    const int c = nodes[w];
    const int par = t.parent[c];
    for (int q = lane; q < nq; q += 32) lp[q] = loc[(size_t)par * nq + q];
    warp_dpow(lane, t.cx[c] - t.cx[par], t.cy[c] - t.cy[par], t.cz[c] - t.cz[par], p, comp, e3, dp);
    for (int tq = lane; tq < nq; tq += 32) {
        const int ct = comp[tq];
        const int tx = cx_(ct), ty = cy_(ct), tz = cz_(ct);
        const int rem = p - (tx + ty + tz);
        double a = 0.0;
        for (int u = 0; u < nT(rem); ++u) {
            const int cu = comp[u];
            a += lp[pidx(tx + cx_(cu), ty + cy_(cu), tz + cz_(cu))] * dp[u];
        }
        loc[(size_t)c * nq + tq] += a;
    }
}

// ---------------------------------------------------------------- L2P
__global__ void k_l2p(const TreeDev t, const double* __restrict__ sx, const double* __restrict__ sy,
                      const double* __restrict__ sz, int64_t n, int p, int f, const double* __restrict__ loc,
                      double* __restrict__ fs) {
    extern __shared__ double smem[];
    const int nq = nT(p);
    int* comp = reinterpret_cast<int*>(smem);
    double* base = smem + (nq + 1) / 2 + 1;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = nq + 32 * 3 * (kMaxP + 1);
    double* lsh = base + wib * per_warp;
    double* e = lsh + nq + lane * 3 * (kMaxP + 1);
    fill_comp(comp, nq);
    __syncthreads();
    const int w = blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= t.num_leaves) return;
    const int leaf = t.leaves[w];
    for (int q = lane; q < nq; q += 32) lsh[q] = loc[(size_t)leaf * nq + q];
    __syncwarp();
    const double cx = t.cx[leaf], cy = t.cy[leaf], cz = t.cz[leaf];
    const int s0 = t.start[leaf], cnt = t.count[leaf];
    const int nf = nT(f);
    for (int k = s0 + lane; k < s0 + cnt; k += 32) {
        scaled_powers(sx[k] - cx, p, e);
        scaled_powers(sy[k] - cy, p, e + (kMaxP + 1));
        scaled_powers(sz[k] - cz, p, e + 2 * (kMaxP + 1));
        for (int tq = 0; tq < nf; ++tq) {
            const int ct = comp[tq];
            const int tx = cx_(ct), ty = cy_(ct), tz = cz_(ct);
            const int rem = p - (tx + ty + tz);
            double a = 0.0;
            for (int u = 0; u < nT(rem); ++u) {
                const int cu = comp[u];
                a += lsh[pidx(tx + cx_(cu), ty + cy_(cu), tz + cz_(cu))] * e[cx_(cu)] * e[(kMaxP + 1) + cy_(cu)] *
                     e[2 * (kMaxP + 1) + cz_(cu)];
            }
            fs[(size_t)tq * n + k] += a;
        }
    }
}

size_t comp_bytes(int nq) { return sizeof(double) * ((nq + 1) / 2 + 1); }

// Terms of the reference's closed-form tensors (src/tensors_recursive.F90:29-62)
// for all components of order <= N, with the int32 Cnij table of
// src/tensors_recursive.F90:64-93 (two's-complement wrap).
void build_ref_terms(int N, std::vector<int32_t>& off, std::vector<uchar4>& abc, std::vector<double>& coef) {
    const int maxo = N, d1 = maxo + 2, d0 = 2 * maxo + 3;
    std::vector<int32_t> C((size_t)d0 * d1 * d1, 0);
    auto at = [&](int nn, int ii, int jj) { return ((size_t)(nn - 1) * d1 + ii) * d1 + jj; };
    for (int nn = 1; nn <= d0; ++nn) C[at(nn, 0, 0)] = 1;
    for (int nn = 1; nn <= d0; ++nn) {
        if (nn % 2 == 0) continue;
        for (int ii = 1; ii <= maxo + 1; ++ii) {
            int k = (ii % 2 != 0) ? ii - 1 : ii;
            for (int jj = 0; jj <= ii; ++jj) {
                if ((ii + jj) % 2 != 0) continue;
                if (jj == 0) {
                    C[at(nn, ii, jj)] = C[at(nn, ii - 1, jj + 1)];
                } else if (jj != ii) {
                    uint32_t a = (uint32_t)(jj + 1) * (uint32_t)C[at(nn, ii - 1, jj + 1)];
                    uint32_t b = (uint32_t)(nn + k) * (uint32_t)C[at(nn, ii - 1, jj - 1)];
                    C[at(nn, ii, jj)] = (int32_t)(a - b);
                    k += 2;
                } else {
                    C[at(nn, ii, jj)] = (int32_t)(0u - (uint32_t)(nn + k) * (uint32_t)C[at(nn, ii - 1, jj - 1)]);
                }
            }
        }
    }
    off.assign(1, 0);
    abc.clear();
    coef.clear();
    for (int nn = 0; nn <= N; ++nn)
        for (int kx = nn; kx >= 0; --kx)
            for (int ky = nn - kx; ky >= 0; --ky) {
                const int kz = nn - kx - ky;
                for (int a = 0; a <= kx; ++a) {
                    const int32_t c1 = C[at(1, kx, a)];
                    if (c1 == 0) continue;
                    for (int b = 0; b <= ky; ++b) {
                        const int32_t c2 = C[at(a + kx + 1, ky, b)];
                        if (c2 == 0) continue;
                        for (int c = 0; c <= kz; ++c) {
                            const int32_t c3 = C[at(a + kx + b + ky + 1, kz, c)];
                            if (c3 == 0) continue;
                            abc.push_back(make_uchar4((unsigned char)a, (unsigned char)b, (unsigned char)c, 0));
                            coef.push_back((double)c1);
                            coef.push_back((double)c2);
                            coef.push_back((double)c3);
                        }
                    }
                }
                off.push_back((int32_t)abc.size());
            }
}

int set_smem(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) FMM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return FMM_OK;
}

}  // namespace

int launch_p2m_m2m(Workspace& ws, const Particles& P, const TreeDev& t, int p, cudaStream_t st) {
    const int nq = nT(p);
    const int m = dim_to_order(P.dim);
    FMM_TRY(ws.mom.ensure(sizeof(double) * (size_t)t.num_nodes * nq));
    double* mom = ws.mom.as<double>();
    {
        const int wpb = 4;
        const size_t sm = comp_bytes(nq) + sizeof(double) * wpb * (nq + 3 * (kMaxP + 1) + 32);
        FMM_TRY(set_smem((const void*)k_p2m, sm));
        count_launches(1);
        k_p2m<<<grid_for(t.num_leaves, wpb), 32 * wpb, sm, st>>>(t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                                  ws.sz.as<double>(), ws.smc.as<double>(), P.n, m, p,
                                                                  mom);
    }
    {
        const int wpb = 4;
        const size_t sm = comp_bytes(nq) + sizeof(double) * wpb * (2 * nq + 3 * (kMaxP + 1));
        FMM_TRY(set_smem((const void*)k_m2m, sm));
        for (int d = t.max_depth - 1; d >= 1; --d) {
            const int lo = t.level_start[d], hi = t.level_start[d + 1];
            if (hi <= lo) continue;
            count_launches(1);
            k_m2m<<<grid_for(hi - lo, wpb), 32 * wpb, sm, st>>>(t, t.level_nodes + lo, hi - lo, p, mom);
        }
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_m2l(Workspace& ws, const TreeDev& t, int p, const Modes& md, cudaStream_t st) {
    const int nq = nT(p), N = 2 * p, nqT = nT(N);
    FMM_TRY(ws.loc.ensure(sizeof(double) * (size_t)t.num_nodes * nq));
    const int ref = md.coef_mode == 0 ? 1 : 0;
    if (ref && ws.term_order != N) {
        std::vector<int32_t> off;
        std::vector<uchar4> abc;
        std::vector<double> coef;
        build_ref_terms(N, off, abc, coef);
        FMM_TRY(ws.term_off.ensure(sizeof(int32_t) * off.size()));
        FMM_TRY(ws.term_abc.ensure(sizeof(uchar4) * std::max<size_t>(1, abc.size())));
        FMM_TRY(ws.term_c.ensure(sizeof(double) * std::max<size_t>(1, coef.size())));
        FMM_CUDA_TRY(cudaMemcpyAsync(ws.term_off.p, off.data(), sizeof(int32_t) * off.size(), cudaMemcpyHostToDevice, st));
        FMM_CUDA_TRY(cudaMemcpyAsync(ws.term_abc.p, abc.data(), sizeof(uchar4) * abc.size(), cudaMemcpyHostToDevice, st));
        FMM_CUDA_TRY(cudaMemcpyAsync(ws.term_c.p, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice, st));
        FMM_CUDA_TRY(cudaStreamSynchronize(st));
        ws.term_order = N;
    }
    if (!ref) return launch_m2l_reduced(ws, t, p, md.precision == 1 || md.precision == 3, st);
    const int per_warp = 2 * nqT + nq + 5 * (N + 1);
    int wpb = (int)std::max<size_t>(1, std::min<size_t>(4, (100 * 1024) / (sizeof(double) * per_warp)));
    const size_t sm = comp_bytes(nqT) + sizeof(double) * wpb * per_warp;
    FMM_TRY(set_smem((const void*)k_m2l_f64, sm));
    count_launches(1);
    k_m2l_f64<<<grid_for(t.num_nodes, wpb), 32 * wpb, sm, st>>>(t, ws.mom.as<double>(), ws.loc.as<double>(), p, ref,
                                                                ws.term_off.as<int32_t>(), ws.term_abc.as<uchar4>(),
                                                                ws.term_c.as<double>());
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_l2l_l2p(Workspace& ws, const Particles& P, const TreeDev& t, int p, int field_order, cudaStream_t st) {
    const int nq = nT(p);
    double* loc = ws.loc.as<double>();
    {
        const int wpb = 4;
        const size_t sm = comp_bytes(nq) + sizeof(double) * wpb * (2 * nq + 3 * (kMaxP + 1));
        FMM_TRY(set_smem((const void*)k_l2l, sm));
        for (int d = 2; d <= t.max_depth; ++d) {
            const int lo = t.level_start[d], hi = t.level_start[d + 1];
            if (hi <= lo) continue;
            count_launches(1);
            k_l2l<<<grid_for(hi - lo, wpb), 32 * wpb, sm, st>>>(t, t.level_nodes + lo, hi - lo, p, loc);
        }
    }
    {
        const int wpb = 2;
        const size_t sm = comp_bytes(nq) + sizeof(double) * wpb * (nq + 32 * 3 * (kMaxP + 1));
        FMM_TRY(set_smem((const void*)k_l2p, sm));
        count_launches(1);
        k_l2p<<<grid_for(t.num_leaves, wpb), 32 * wpb, sm, st>>>(t, ws.sx.as<double>(), ws.sy.as<double>(),
                                                                  ws.sz.as<double>(), P.n, p, field_order, loc,
                                                                  ws.fsorted.as<double>());
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

// Reference-mode M2L (FP64): the reference's own closed-form tensors with the
// int32 Cnij table (src/tensors_recursive.F90:29-135) over the full Cartesian
// bases, L_f(i) += sum_s (-1)^(|s|+1) M'_s(j) T_{s+f}(c_i - c_j)
// (src/fmm.F90:826-882), with M'_s = M_s / s! the scaled moments of
// translate.cu.  The exact-coefficient modes use the reduced-basis M2L
// (m2l.cu, m2l_gemm.cu) instead.
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

}  // namespace fmm

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

// The tensor T_c(X, Y, Z) of every component c < nT(N) in the warp's shared
// memory: the reference's closed form with its Cnij table (ref) or the Hermite
// recursion (exact).  Returns TA or TB, whichever holds the result.
__device__ double* warp_tensor(double X, double Y, double Z, int N, int ref, const int* __restrict__ comp,
                               double* TA, double* TB, double* gsh, double* yp, double* zp, double* ir,
                               const int32_t* __restrict__ term_off, const uchar4* __restrict__ term_abc,
                               const double* __restrict__ term_c, int lane) {
    const int nqT = nT(N);
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
    return T;
}

__global__ void k_m2l_f64(const TreeDev t, const double* __restrict__ mom, double* __restrict__ loc, int p, int ref,
                          const int32_t* __restrict__ term_off, const uchar4* __restrict__ term_abc,
                          const double* __restrict__ term_c, int accumulate) {
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
        // the source cell of a periodic image is displaced by t.shift (0 otherwise)
        const double X = __dsub_rn(cxi, __dadd_rn(t.cx[j], t.shift[0]));
        const double Y = __dsub_rn(cyi, __dadd_rn(t.cy[j], t.shift[1]));
        const double Z = __dsub_rn(czi, __dadd_rn(t.cz[j], t.shift[2]));
        for (int s = lane; s < nq; s += 32) {
            const double v = mom[(size_t)j * nq + s];
            ms[s] = ((order_of(s) + 1) % 2) ? -v : v;  // (-1)^(|s|+1) M'_s
        }
        double* T = warp_tensor(X, Y, Z, N, ref, comp, TA, TB, gsh, yp, zp, ir, term_off, term_abc, term_c, lane);
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
        if (fq < nq) {
            double* L = loc + (size_t)i * nq + fq;
            *L = accumulate ? *L + acc[r] : acc[r];
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

// Closed-form tensor terms of the reference at order N (ref mode), once per order.
int ensure_ref_terms(Workspace& ws, int N, cudaStream_t st) {
    if (ws.term_order == N) return FMM_OK;
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
    return FMM_OK;
}

int launch_m2l_pairwise(Workspace& ws, const TreeDev& t, int p, const Modes& md, bool accumulate, cudaStream_t st) {
    const int nq = nT(p), N = 2 * p, nqT = nT(N);
    FMM_TRY(ws.loc.ensure(sizeof(double) * (size_t)t.num_nodes * nq));
    const int ref = md.coef_mode == 0 ? 1 : 0;
    if (ref) FMM_TRY(ensure_ref_terms(ws, N, st));
    const int per_warp = 2 * nqT + nq + 5 * (N + 1);
    int wpb = (int)std::max<size_t>(1, std::min<size_t>(4, (100 * 1024) / (sizeof(double) * per_warp)));
    const size_t sm = comp_bytes(nqT) + sizeof(double) * wpb * per_warp;
    FMM_TRY(set_smem((const void*)k_m2l_f64, sm));
    count_launches(1);
    k_m2l_f64<<<grid_for(t.num_nodes, wpb), 32 * wpb, sm, st>>>(t, ws.mom.as<double>(), ws.loc.as<double>(), p, ref,
                                                                ws.term_off.as<int32_t>(), ws.term_abc.as<uchar4>(),
                                                                ws.term_c.as<double>(), accumulate ? 1 : 0);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_m2l(Workspace& ws, const TreeDev& t, int p, const Modes& md, cudaStream_t st) {
    if (md.coef_mode != 0) return launch_m2l_reduced(ws, t, p, md.precision == 1 || md.precision == 3, st);
    return launch_m2l_pairwise(ws, t, p, md, false, st);
}

// ---------------------------------------------------------------- periodic
// The lattice beyond the 27 explicit images (src/fmm.F90:884-952), for the
// root's local expansion.  Level multipoles, scaled like the cell moments
// (M'_t = M_t / t!): S_0 is the root's with its charge removed (the
// reference forces charge neutrality), and S_l = S_(l-1) plus the 26 copies
// of S_(l-1) shifted by H (3^(l-1) a), a != 0, in the reference's order of a.
// One block; S_0 .. S_(L-1) are written to S (L x nq).
__global__ void k_lattice_moments(int p, int L, const double* __restrict__ root_mom, const Box9 H,
                                  double* __restrict__ S) {
    extern __shared__ double sh[];
    const int nq = nT(p), P1 = p + 1;
    double* src = sh;
    double* dst = src + nq;
    double* e = dst + nq;  // scaled powers d^u / u! per axis, 3 x (p + 1)
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        const double v = q == 0 ? 0.0 : root_mom[q];
        src[q] = v;
        S[q] = v;
    }
    __syncthreads();
    double three_l = 1.0;
    for (int l = 1; l < L; ++l) {
        three_l *= 3.0;  // 3^l, exact
        for (int q = threadIdx.x; q < nq; q += blockDim.x) dst[q] = src[q];
        __syncthreads();
        for (int ai = -1; ai <= 1; ++ai)
            for (int aj = -1; aj <= 1; ++aj)
                for (int ak = -1; ak <= 1; ++ak) {
                    if (ai == 0 && aj == 0 && ak == 0) continue;
                    if (threadIdx.x < 3) {
                        const int ax = threadIdx.x;
                        // d_aijk = matmul(H, a 3^l) / 3 (fmm.F90:920-923)
                        const double v = __dadd_rn(__dadd_rn(__dmul_rn(H.h[ax], ai * three_l),
                                                             __dmul_rn(H.h[3 + ax], aj * three_l)),
                                                   __dmul_rn(H.h[6 + ax], ak * three_l));
                        const double d = __ddiv_rn(v, 3.0);
                        double pw = 1.0, fact = 1.0;
                        for (int u = 0; u <= p; ++u) {
                            e[ax * P1 + u] = pw / fact;
                            pw *= d;
                            fact *= (double)(u + 1);
                        }
                    }
                    __syncthreads();
                    for (int t = threadIdx.x; t < nq; t += blockDim.x) {
                        const int tx = comp_x(t), ty = comp_y(t), tz = comp_z(t), to = tx + ty + tz;
                        double acc = 0.0;
                        for (int so = 0; so <= to; ++so)
                            for (int sx = min(so, tx); sx >= 0; --sx)
                                for (int sy = min(so - sx, ty); sy >= 0; --sy) {
                                    const int sz = so - sx - sy;
                                    if (sz > tz) continue;
                                    acc += e[tx - sx] * e[P1 + ty - sy] * e[2 * P1 + tz - sz] * src[pidx(sx, sy, sz)];
                                }
                        dst[t] += acc;
                    }
                    __syncthreads();
                }
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            src[q] = dst[q];
            S[(size_t)l * nq + q] = dst[q];
        }
        __syncthreads();
    }
}

// Level l (1 .. L): the 702 copies of S_(l-1) at H (3^l a + 3^(l-1) b),
// a != 0 and b in {-1,0,1}^3, evaluated at the root centre like the
// reference's multipole_field call (tensors at R = the copy's position,
// src/fmm.F90:929-943).  Block (l-1, slice) sums a slice of the copies;
// partial sums go to C ((L x slices) x nq).  In exact mode the tensors are
// evaluated at R 2^-k (k ~ l log2 3, an exact scaling) and the moments and
// results rescaled by the matching powers of two, so the recursion's r^-(4p+1)
// does not underflow at the far levels; ref mode follows the reference's
// closed form unscaled.
constexpr int kLatticeSlices = 16;

__global__ void k_lattice_m2l(int p, int L, int ref, const double* __restrict__ S, const Box9 H,
                              const int32_t* __restrict__ term_off, const uchar4* __restrict__ term_abc,
                              const double* __restrict__ term_c, double* __restrict__ C) {
    extern __shared__ double smem[];
    const int nq = nT(p), N = 2 * p, nqT = nT(N);
    int* comp = reinterpret_cast<int*>(smem);
    double* base = smem + (nqT + 1) / 2 + 1;
    const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = 2 * nqT + nq + 5 * (N + 1);
    double* red = base + nw * per_warp;  // nw x nq
    double* TA = base + wib * per_warp;
    double* TB = TA + nqT;
    double* ms = TB + nqT;
    double* gsh = ms + nq;
    double* yp = gsh + (N + 1);
    double* zp = yp + (N + 1);
    double* ir = zp + (N + 1);
    fill_comp(comp, nqT);
    const int l = blockIdx.x + 1, slice = blockIdx.y;
    const int ksc = ref ? 0 : (int)floor(l * 1.5849625007211563);  // log2(3)
    const double* Sl = S + (size_t)(l - 1) * nq;
    for (int s = lane; s < nq; s += 32) {
        const double v = Sl[s];
        ms[s] = ldexp(((order_of(s) + 1) % 2) ? -v : v, -ksc * order_of(s));  // (-1)^(|s|+1) M'_s 2^(-k|s|)
    }
    __syncthreads();
    double three_l = 1.0;
    for (int k = 0; k < l; ++k) three_l *= 3.0;
    const double three_lm = three_l / 3.0;
    int fcomp[kMaxNPL];
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) fcomp[r] = (lane + 32 * r < nq) ? comp[lane + 32 * r] : 0;
    double acc[kMaxNPL];
#pragma unroll
    for (int r = 0; r < kMaxNPL; ++r) acc[r] = 0.0;
    for (int k = slice * nw + wib; k < 26 * 27; k += kLatticeSlices * nw) {
        int ka = k / 27, kb = k % 27;
        if (ka >= 13) ++ka;  // skip a = 0 (index 13 of the 27 in i,j,k order)
        const int ai = ka / 9 - 1, aj = (ka / 3) % 3 - 1, ak = ka % 3 - 1;
        const int bi = kb / 9 - 1, bj = (kb / 3) % 3 - 1, bk = kb % 3 - 1;
        double pos[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const double da = __dadd_rn(__dadd_rn(__dmul_rn(H.h[ax], ai * three_l), __dmul_rn(H.h[3 + ax], aj * three_l)),
                                        __dmul_rn(H.h[6 + ax], ak * three_l));
            const double db = __dadd_rn(__dadd_rn(__dmul_rn(H.h[ax], bi * three_lm), __dmul_rn(H.h[3 + ax], bj * three_lm)),
                                        __dmul_rn(H.h[6 + ax], bk * three_lm));
            pos[ax] = ldexp(__dadd_rn(da, db), -ksc);
        }
        double* T = warp_tensor(pos[0], pos[1], pos[2], N, ref, comp, TA, TB, gsh, yp, zp, ir, term_off, term_abc,
                                term_c, lane);
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
    for (int r = 0; r < kMaxNPL; ++r)
        if (lane + 32 * r < nq) red[wib * nq + lane + 32 * r] = acc[r];
    __syncthreads();
    for (int f = threadIdx.x; f < nq; f += blockDim.x) {
        double v = 0.0;
        for (int w = 0; w < nw; ++w) v += red[w * nq + f];
        C[((size_t)(l - 1) * kLatticeSlices + slice) * nq + f] = ldexp(v, -ksc * (order_of(f) + 1));
    }
}

// Adds the levels' contributions to the root's local expansion in order and
// stops after the first level whose contribution (without its first
// component) has a norm below tol, as the reference does (fmm.F90:944-950);
// levels_used receives the number of levels added.
__global__ void k_lattice_apply(int nq, int L, const double* __restrict__ C, double* __restrict__ loc_root,
                                double tol, int* levels_used) {
    __shared__ double lev[kMaxNPL * 32];
    __shared__ int stop;
    const int lane = threadIdx.x;
    int used = 0;
    for (int l = 0; l < L; ++l) {
        for (int f = lane; f < nq; f += 32) {
            double v = 0.0;
            for (int sl = 0; sl < kLatticeSlices; ++sl) v += C[((size_t)l * kLatticeSlices + sl) * nq + f];
            lev[f] = v;
            loc_root[f] += v;
        }
        __syncwarp();
        if (lane == 0) {
            // NORM2 as the scaled sum of squares
            double scale = 0.0, ssq = 1.0;
            for (int f = 1; f < nq; ++f) {
                const double v = lev[f];
                if (v != 0.0) {
                    const double ax = fabs(v);
                    if (scale < ax) {
                        const double t = scale / ax;
                        ssq = 1.0 + (ssq * t) * t;
                        scale = ax;
                    } else {
                        const double t = ax / scale;
                        ssq = ssq + t * t;
                    }
                }
            }
            stop = (scale * sqrt(ssq) < tol) ? 1 : 0;
        }
        __syncwarp();
        ++used;
        if (stop) break;
    }
    if (lane == 0) *levels_used = used;
}

// Surface term of the periodic sum (src/fmm.F90:954-979), on the field in
// sorted order: phi-column += 4 pi (D . x) / 3V + 2 pi tr(Q) / 3V and the
// order-1 columns += 4 pi D / 3V, with D and tr(Q) the root's dipole and
// quadrupole trace.  Ref mode keeps the reference's constant for pi and its
// cofactor expansion of the volume; exact mode the true ones.
__global__ void k_dipole_fix(int64_t n, int f, const double* __restrict__ sx, const double* __restrict__ sy,
                             const double* __restrict__ sz, const double* __restrict__ root_mom, const Box9 H,
                             int ref, double* __restrict__ fs) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    auto h = [&](int i, int j) { return H.h[(j - 1) * 3 + (i - 1)]; };  // h(i, j), column-major
    double vol;
    if (ref)
        vol = h(1, 1) * (h(2, 2) * h(3, 3) - h(2, 3) * h(3, 2)) - h(1, 2) * (h(2, 1) * h(3, 3) - h(2, 3) * h(3, 1)) +
              h(1, 3) * (h(1, 2) * h(3, 2) - h(2, 2) * h(3, 1));
    else
        vol = h(1, 1) * (h(2, 2) * h(3, 3) - h(2, 3) * h(3, 2)) - h(1, 2) * (h(2, 1) * h(3, 3) - h(2, 3) * h(3, 1)) +
              h(1, 3) * (h(2, 1) * h(3, 2) - h(2, 2) * h(3, 1));
    const double pi = ref ? 3.14159265359 : 3.141592653589793;
    const double dx = root_mom[1], dy = root_mom[2], dz = root_mom[3];
    // raw second moments are 2! times the scaled ones
    const double tr = 2.0 * root_mom[4] + 2.0 * root_mom[7] + 2.0 * root_mom[9];
    const double dot = dx * sx[k] + dy * sy[k] + dz * sz[k];
    fs[k] = fs[k] + 4.0 * pi * dot / (3.0 * vol) + 2.0 * pi * tr / (3.0 * vol);
    if (f >= 1) {
        const double c = 4.0 * pi / (3.0 * vol);
        fs[(size_t)1 * n + k] += c * dx;
        fs[(size_t)2 * n + k] += c * dy;
        fs[(size_t)3 * n + k] += c * dz;
    }
}

int launch_periodic_lattice(Workspace& ws, const TreeDev& t, int p, int f, const Modes& md, const Box9& H,
                            double* d_fs, int* d_levels, cudaStream_t st) {
    constexpr int L = 50;  // the reference's limit of levels
    const int nq = nT(p), N = 2 * p, nqT = nT(N);
    const int ref = md.coef_mode == 0 ? 1 : 0;
    if (ref) FMM_TRY(ensure_ref_terms(ws, N, st));
    FMM_TRY(ws.lattice.ensure(sizeof(double) * ((size_t)L * nq + (size_t)L * kLatticeSlices * nq)));
    double* S = ws.lattice.as<double>();
    double* C = S + (size_t)L * nq;
    const double* root_mom = ws.mom.as<double>();  // the root is node 0
    {
        const size_t sm = sizeof(double) * (2 * nq + 3 * (p + 1));
        FMM_TRY(set_smem((const void*)k_lattice_moments, sm));
        count_launches(1);
        k_lattice_moments<<<1, 256, sm, st>>>(p, L, root_mom, H, S);
    }
    {
        const int per_warp = 2 * nqT + nq + 5 * (N + 1);
        int nw = (int)std::max<size_t>(1, std::min<size_t>(4, (100 * 1024) / (sizeof(double) * (per_warp + nq))));
        const size_t sm = comp_bytes(nqT) + sizeof(double) * nw * (per_warp + nq);
        FMM_TRY(set_smem((const void*)k_lattice_m2l, sm));
        count_launches(1);
        k_lattice_m2l<<<dim3(L, kLatticeSlices), 32 * nw, sm, st>>>(p, L, ref, S, H, ws.term_off.as<int32_t>(),
                                                                     ws.term_abc.as<uchar4>(),
                                                                     ws.term_c.as<double>(), C);
    }
    count_launches(1);
    k_lattice_apply<<<1, 32, 0, st>>>(nq, L, C, ws.loc.as<double>(), 1.0e-8, d_levels);
    count_launches(1);
    k_dipole_fix<<<grid_for(t.n, 256), 256, 0, st>>>(t.n, f, ws.sx.as<double>(), ws.sy.as<double>(),
                                                      ws.sz.as<double>(), root_mom, H, ref, d_fs);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

}  // namespace fmm

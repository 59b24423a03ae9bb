// Pair interaction math shared by the direct-sum and near-field kernels.
//
// The reference evaluates interaction tensors with a closed form for the
// undamped kernel (src/tensors_recursive.F90:95-135) and with generated
// straight-line code for the damped ones (src/tensors_damped_*.F90).  Here
// every kernel goes through one path:
//   1. radial functions g_j(r) = (r^-1 d/dr)^j phi(r), j = 0..N, for the
//      kernel phi (1/r, Thole, AMOEBA, erf);
//   2. the Cartesian derivative tensor T_{tuv} = d^t/dx^t d^u/dy^u d^v/dz^v phi
//      of every order <= N from the g_j by the Hermite-type recursion
//        R^(j)_{t+1,u,v} = t R^(j+1)_{t-1,u,v} + X R^(j+1)_{t,u,v},
//      R^(j)_{000} = g_j, T = R^(0) (done in place, highest level first);
//   3. the contraction of the reference's multipole_field
//      (src/fmm.F90:596-620): F_f += sum_s c_s M_s T_{s+f}, where the
//      source coefficients c_s = (-1)^(|s|+1) / (sx! sy! sz!) are folded into
//      the multipoles once per particle.
// Everything is templated on the multipole order M and field order F, so the
// compiler unrolls it into straight-line register code.
#pragma once

#include <math.h>

#include "common.cuh"
#include "series_tables.h"

namespace fmm {

#define FMM_INV_ODD_N 64
#ifdef __CUDACC__
__constant__ double cInvOdd[FMM_INV_ODD_N] = {
#define X(i) 1.0 / (2.0 * (i) + 1.0),
    X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15)
    X(16) X(17) X(18) X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27) X(28) X(29) X(30) X(31)
    X(32) X(33) X(34) X(35) X(36) X(37) X(38) X(39) X(40) X(41) X(42) X(43) X(44) X(45) X(46) X(47)
    X(48) X(49) X(50) X(51) X(52) X(53) X(54) X(55) X(56) X(57) X(58) X(59) X(60) X(61) X(62) X(63)
#undef X
};
__constant__ double cTholeSeries[FMM_SER_JMAX + 1][FMM_SER_KT + 1] = FMM_THOLE_SERIES_INIT;
__constant__ double cAmoebaSeries[FMM_SER_JMAX + 1][FMM_SER_KA + 1] = FMM_AMOEBA_SERIES_INIT;
__constant__ double cAmoebaQ[FMM_SER_JMAX + 1][FMM_SER_JMAX] = FMM_AMOEBA_Q_INIT;
__constant__ float cAmoebaQF[FMM_SER_JMAX + 1][FMM_SER_JMAX] = FMM_AMOEBA_Q_INIT;
// interval expansions (FP32 kernels): lanes index them by their own
// interval, so they live in global memory rather than the constant bank;
// rows are read as float4s
__device__ __align__(16) const float gTholeTay[FMM_SER_JMAX + 1][FMM_THOLE_NC][FMM_TAY_N] = FMM_THOLE_TAY_INIT;
__device__ __align__(16) const float gAmoebaTay[FMM_SER_JMAX + 1][FMM_AMOEBA_NC][FMM_TAY_N] = FMM_AMOEBA_TAY_INIT;
#endif
static const double hTholeTay[FMM_SER_JMAX + 1][FMM_THOLE_NC][FMM_TAY_N] = FMM_THOLE_TAY_INIT;
static const double hAmoebaTay[FMM_SER_JMAX + 1][FMM_AMOEBA_NC][FMM_TAY_N] = FMM_AMOEBA_TAY_INIT;
static const double hTholeSeries[FMM_SER_JMAX + 1][FMM_SER_KT + 1] = FMM_THOLE_SERIES_INIT;
static const double hAmoebaSeries[FMM_SER_JMAX + 1][FMM_SER_KA + 1] = FMM_AMOEBA_SERIES_INIT;
static const double hAmoebaQ[FMM_SER_JMAX + 1][FMM_SER_JMAX] = FMM_AMOEBA_Q_INIT;

// Per-precision math and the switch-over points between the series and the
// closed forms (chosen so the closed form's cancellation stays below the
// precision's rounding; checked against high-precision values in the tests).
template <typename R>
struct Real;

template <>
struct Real<double> {
    static constexpr double kTholeX = 0.5;   // series for a*r below this
    static constexpr int kTholeK = 18;       // series terms used
    static constexpr double kAmoebaU = 0.5;  // series for (a r)^3 below this
    static constexpr int kAmoebaK = 16;
    static constexpr double kErfS = 3.0;     // Boys series for a r^2 below this
    static constexpr int kErfK = 40;
    static constexpr bool kTay = false;      // interval tables unused in FP64
    __host__ __device__ static __forceinline__ void thole_row(int, int, double*) {}
    __host__ __device__ static __forceinline__ void amoeba_row(int, int, double*) {}
    __host__ __device__ static __forceinline__ double rsqrt_(double x) {
#ifdef __CUDA_ARCH__
        return ::rsqrt(x);
#else
        return 1.0 / ::sqrt(x);
#endif
    }
    __host__ __device__ static __forceinline__ double exp_(double x) { return ::exp(x); }
    __host__ __device__ static __forceinline__ double expc_(double x) { return ::exp(x); }
    __host__ __device__ static __forceinline__ double erf_(double x) { return ::erf(x); }
    __host__ __device__ static __forceinline__ double sqrt_(double x) { return ::sqrt(x); }
    __host__ __device__ static __forceinline__ double inv_odd(int i) {
#ifdef __CUDA_ARCH__
        return cInvOdd[i];
#else
        return 1.0 / (2.0 * i + 1.0);
#endif
    }
    __host__ __device__ static __forceinline__ double thole(int j, int k) {
#ifdef __CUDA_ARCH__
        return cTholeSeries[j][k];
#else
        return hTholeSeries[j][k];
#endif
    }
    __host__ __device__ static __forceinline__ double amoeba(int j, int k) {
#ifdef __CUDA_ARCH__
        return cAmoebaSeries[j][k];
#else
        return hAmoebaSeries[j][k];
#endif
    }
    __host__ __device__ static __forceinline__ double amoebaQ(int j, int d) {
#ifdef __CUDA_ARCH__
        return cAmoebaQ[j][d];
#else
        return hAmoebaQ[j][d];
#endif
    }
};

template <>
struct Real<float> {
    // interval tables below 3 (Thole, x = a r) and 4 (AMOEBA, u = (a r)^3):
    // the series on [0, 1), re-centred expansions on the unit intervals
    // above; closed forms beyond
    static constexpr bool kTay = true;
    static constexpr float kTholeHi = (float)FMM_THOLE_NC;
    static constexpr float kAmoebaHi = (float)FMM_AMOEBA_NC;
    static_assert(FMM_TAY_N % 4 == 0, "interval rows are read as float4");
    __host__ __device__ static __forceinline__ void thole_row(int j, int c, float* b) {
#ifdef __CUDA_ARCH__
        const float4* r = reinterpret_cast<const float4*>(&gTholeTay[j][c][0]);
#pragma unroll
        for (int v = 0; v < FMM_TAY_N / 4; ++v) {
            const float4 w = __ldg(r + v);
            b[4 * v] = w.x;
            b[4 * v + 1] = w.y;
            b[4 * v + 2] = w.z;
            b[4 * v + 3] = w.w;
        }
#else
        for (int n = 0; n < FMM_TAY_N; ++n) b[n] = (float)hTholeTay[j][c][n];
#endif
    }
    __host__ __device__ static __forceinline__ void amoeba_row(int j, int c, float* b) {
#ifdef __CUDA_ARCH__
        const float4* r = reinterpret_cast<const float4*>(&gAmoebaTay[j][c][0]);
#pragma unroll
        for (int v = 0; v < FMM_TAY_N / 4; ++v) {
            const float4 w = __ldg(r + v);
            b[4 * v] = w.x;
            b[4 * v + 1] = w.y;
            b[4 * v + 2] = w.z;
            b[4 * v + 3] = w.w;
        }
#else
        for (int n = 0; n < FMM_TAY_N; ++n) b[n] = (float)hAmoebaTay[j][c][n];
#endif
    }
    static constexpr float kErfS = 6.0f;
    static constexpr int kErfK = 36;
    __host__ __device__ static __forceinline__ float rsqrt_(float x) {
#ifdef __CUDA_ARCH__
        return ::rsqrtf(x);
#else
        return 1.0f / ::sqrtf(x);
#endif
    }
    __host__ __device__ static __forceinline__ float exp_(float x) { return ::expf(x); }
    // e^x for the closed forms of the damped numerators (x <= -3): there it
    // scales a correction of at most ~0.3 of the numerator's constant term,
    // so the fast intrinsic's error (~1e-6 relative at |x| ~ 20) stays below
    // 1e-7 of the numerator
    __host__ __device__ static __forceinline__ float expc_(float x) {
#ifdef __CUDA_ARCH__
        return __expf(x);
#else
        return ::expf(x);
#endif
    }
    __host__ __device__ static __forceinline__ float erf_(float x) { return ::erff(x); }
    __host__ __device__ static __forceinline__ float sqrt_(float x) { return ::sqrtf(x); }
    __host__ __device__ static __forceinline__ float inv_odd(int i) {
#ifdef __CUDA_ARCH__
        return (float)cInvOdd[i];
#else
        return 1.0f / (2.0f * i + 1.0f);
#endif
    }
    __host__ __device__ static __forceinline__ float amoebaQ(int j, int d) {
#ifdef __CUDA_ARCH__
        return cAmoebaQF[j][d];
#else
        return (float)hAmoebaQ[j][d];
#endif
    }
};

__host__ __device__ constexpr double dfact_odd(int j) {  // (2j-1)!!, (-1)!! = 1
    double p = 1.0;
    for (int i = 1; i <= j; ++i) p *= (double)(2 * i - 1);
    return p;
}

// Interval of v in the FP32 tables and the offset from its centre (the
// series on [0, 1) has centre 0, the interval [c, c + 1) above it c + 1/2).
template <typename R>
__host__ __device__ __forceinline__ R table_offset(R v, int& c) {
    c = (int)v;
    return c == 0 ? v : v - ((R)c + (R)0.5);
}

// Horner sum of one table row at offset t.
template <typename R>
__host__ __device__ __forceinline__ R table_horner(const R* b, R t) {
    R acc = b[FMM_TAY_N - 1];
#pragma unroll
    for (int k = FMM_TAY_N - 2; k >= 0; --k) acc = acc * t + b[k];
    return acc;
}

// g_j(r), j = 0..N, of the kernel `damp` at squared distance r2 and pair
// damping factor a (the product of the two particles' factors).
template <int N, typename R>
__host__ __device__ __forceinline__ void radial_g_ir(int damp, R r2, R ir, R a, R* g, R eps = (R)0);

template <int N, typename R>
__host__ __device__ __forceinline__ void radial_g(int damp, R r2, R a, R* g) {
    radial_g_ir<N, R>(damp, r2, Real<R>::rsqrt_(r2), a, g);
}

// Same, with 1/r supplied by the caller (e.g. a refined FP32 value) and,
// optionally, the relative error eps of that value (1/r = ir (1 + eps)):
// the powers r^-(2j+1) then carry the correction (2j+1) eps, which keeps the
// error of a rounded ir from growing with the tensor order.
template <int N, typename R>
__host__ __device__ __forceinline__ void radial_g_ir(int damp, R r2, R ir, R a, R* g, R eps) {
    using RT = Real<R>;
    const R ir2 = ir * ir;
    if (damp == DAMP_NONE) {
        g[0] = ir;
#pragma unroll
        for (int j = 1; j <= N; ++j) g[j] = -(R)(2 * j - 1) * g[j - 1] * ir2;
#pragma unroll
        for (int j = 0; j <= N; ++j) g[j] += g[j] * ((R)(2 * j + 1) * eps);
        return;
    }
    if (damp == DAMP_ERF) {
        // g_j = (-1)^j sqrt(a) (2a)^j (2/sqrt(pi)) F_j(a r^2), F_j the Boys function
        const R s = a * r2;
        const R es = RT::exp_(-s);
        R Fb[N + 1];
        if (s < RT::kErfS) {
            R term = (R)(1.0 / (2 * N + 1)), sum = term;
            const R two_s = s + s;
#pragma unroll 1
            for (int k = 1; k <= RT::kErfK; ++k) {
                term = term * two_s * RT::inv_odd(N + k);
                sum += term;
            }
            Fb[N] = es * sum;
#pragma unroll
            for (int j = N - 1; j >= 0; --j) Fb[j] = (two_s * Fb[j + 1] + es) * (R)(1.0 / (2 * j + 1));
        } else {
            const R rs = RT::sqrt_(s);
            Fb[0] = (R)0.88622692545275801365 * RT::erf_(rs) / rs;  // sqrt(pi)/2
            const R i2s = (R)0.5 / s;
#pragma unroll
            for (int j = 0; j < N; ++j) Fb[j + 1] = ((R)(2 * j + 1) * Fb[j] - es) * i2s;
        }
        R pre = RT::sqrt_(a) * (R)1.12837916709551257390;  // 2/sqrt(pi)
        const R twoa = a + a;
#pragma unroll
        for (int j = 0; j <= N; ++j) {
            g[j] = (j % 2 ? -pre : pre) * Fb[j];
            pre *= twoa;
        }
        return;
    }
    R num[N + 1];
    if (damp == DAMP_THOLE) {
        const R x = a * (r2 * ir);
        bool closed;
        if constexpr (RT::kTay) {
            closed = !(x < RT::kTholeHi);
            if (!closed) {
                int c;
                const R t = table_offset(x, c);
#pragma unroll
                for (int j = 0; j <= N; ++j) {
                    R b[FMM_TAY_N];
                    RT::thole_row(j, c, b);
                    num[j] = table_horner(b, t);
                }
            }
        } else {
            closed = !(x < RT::kTholeX);
            if (!closed) {
#pragma unroll
                for (int j = 0; j <= N; ++j) {
                    R acc = RT::thole(j, RT::kTholeK);
#pragma unroll 1
                    for (int k = RT::kTholeK - 1; k >= 0; --k) acc = acc * x + RT::thole(j, k);
                    num[j] = acc;
                }
            }
        }
        if (closed && sizeof(R) == 8 && x > (R)100) {
            // FP64, far beyond the damping range: e^{-x} P(x) is below 1e-29
            // of the undamped value, so the sum rounds to it exactly
            num[0] = (R)1;
#pragma unroll
            for (int j = 1; j <= N; ++j) num[j] = (R)((j % 2 ? -1.0 : 1.0) * dfact_odd(j));
        } else if (closed) {
            const R e = RT::expc_(-x);
            const R x2 = x * x;
            R ym1 = (R)1, y0 = -((R)1 + x);  // y_0, y_1 (Yukawa numerators)
            num[0] = (R)1 - e * ((R)1 + (R)0.5 * x);
#pragma unroll
            for (int j = 1; j <= N; ++j) {
                const R P = y0 - (R)0.5 * x2 * ym1;
                num[j] = (R)((j % 2 ? -1.0 : 1.0) * dfact_odd(j)) - e * P;
                const R yn = x2 * ym1 - (R)(2 * j + 1) * y0;
                ym1 = y0;
                y0 = yn;
            }
        }
    } else {  // AMOEBA: T0 = 0, g_1 = -(1 - e^{-u}) / r^3, u = (a r)^3
        const R x = a * (r2 * ir);
        const R u = x * x * x;
        num[0] = (R)0;
        bool closed;
        if constexpr (RT::kTay) {
            closed = !(u < RT::kAmoebaHi);
            if (!closed) {
                int c;
                const R t = table_offset(u, c);
#pragma unroll
                for (int j = 1; j <= N; ++j) {
                    R b[FMM_TAY_N];
                    RT::amoeba_row(j, c, b);
                    num[j] = table_horner(b, t);
                }
            }
        } else {
            closed = !(u < RT::kAmoebaU);
            if (!closed) {
#pragma unroll
                for (int j = 1; j <= N; ++j) {
                    R acc = RT::amoeba(j, RT::kAmoebaK);
#pragma unroll 1
                    for (int k = RT::kAmoebaK - 1; k >= 0; --k) acc = acc * u + RT::amoeba(j, k);
                    num[j] = acc;
                }
            }
        }
        if (closed && sizeof(R) == 8 && u > (R)80) {
            // FP64, far beyond the damping range: e^{-u} q(u) is below 1e-25
            // of the undamped value, so the sum rounds to it exactly
#pragma unroll
            for (int j = 1; j <= N; ++j) num[j] = (R)((j % 2 ? -1.0 : 1.0) * dfact_odd(j));
        } else if (closed) {
            const R e = RT::expc_(-u);
#pragma unroll
            for (int j = 1; j <= N; ++j) {
                R q = RT::amoebaQ(j, j - 1);
#pragma unroll
                for (int d = j - 2; d >= 0; --d) q = q * u + RT::amoebaQ(j, d);
                num[j] = (R)((j % 2 ? -1.0 : 1.0) * dfact_odd(j)) + e * q;
            }
        }
    }
    R irp = ir;
#pragma unroll
    for (int j = 0; j <= N; ++j) {
        const R v = num[j] * irp;
        g[j] = v + v * ((R)(2 * j + 1) * eps);
        irp *= ir2;
    }
}

// Cartesian derivative tensor of all orders <= N from g_0..g_N (in place).
template <int N, typename R>
__host__ __device__ __forceinline__ void md_tensor(R X, R Y, R Z, const R* g, R* T) {
    T[0] = g[N];
#pragma unroll
    for (int j = N - 1; j >= 0; --j) {
#pragma unroll
        for (int k = N - j; k >= 1; --k) {
#pragma unroll
            for (int tx = k; tx >= 0; --tx) {
#pragma unroll
                for (int ty = k - tx; ty >= 0; --ty) {
                    const int tz = k - tx - ty;
                    R v;
                    if (tx > 0) {
                        v = X * T[pidx(tx - 1, ty, tz)];
                        if (tx > 1) v += (R)(tx - 1) * T[pidx(tx - 2, ty, tz)];
                    } else if (ty > 0) {
                        v = Y * T[pidx(tx, ty - 1, tz)];
                        if (ty > 1) v += (R)(ty - 1) * T[pidx(tx, ty - 2, tz)];
                    } else {
                        v = Z * T[pidx(tx, ty, tz - 1)];
                        if (tz > 1) v += (R)(tz - 1) * T[pidx(tx, ty, tz - 2)];
                    }
                    T[pidx(tx, ty, tz)] = v;
                }
            }
        }
        T[0] = g[j];
    }
}

// Source coefficient c_s = (-1)^(|s|+1) / (sx! sy! sz!) of the reference's
// contraction (taylor * symfac in src/fmm.F90:598-615).
__host__ __device__ constexpr double src_coef(int s) {
    return ((order_of(s) + 1) % 2 ? -1.0 : 1.0) / (cfact(comp_x(s)) * cfact(comp_y(s)) * cfact(comp_z(s)));
}

// acc_f += sum_s Mc_s T_{s+f}; Mc already carries src_coef.
template <int M, int F, typename R>
__host__ __device__ __forceinline__ void contract(const R* T, const R* Mc, R* acc) {
#pragma unroll
    for (int fo = 0; fo <= F; ++fo)
#pragma unroll
        for (int fx = fo; fx >= 0; --fx)
#pragma unroll
            for (int fy = fo - fx; fy >= 0; --fy) {
                const int fz = fo - fx - fy;
                R a = acc[pidx(fx, fy, fz)];
#pragma unroll
                for (int so = 0; so <= M; ++so)
#pragma unroll
                    for (int sx = so; sx >= 0; --sx)
#pragma unroll
                        for (int sy = so - sx; sy >= 0; --sy) {
                            const int sz = so - sx - sy;
                            a += Mc[pidx(sx, sy, sz)] * T[pidx(sx + fx, sy + fy, sz + fz)];
                        }
                acc[pidx(fx, fy, fz)] = a;
            }
}

// Field of one source at displacement (dx, dy, dz) = target - source.
template <int M, int F, typename R>
__host__ __device__ __forceinline__ void pair_field(R dx, R dy, R dz, R a, int damp, const R* Mc, R* acc) {
    constexpr int N = M + F;
    const R r2 = dx * dx + dy * dy + dz * dz;
    R g[N + 1];
    radial_g<N, R>(damp, r2, a, g);
    R T[nT(N)];
    md_tensor<N, R>(dx, dy, dz, g, T);
    contract<M, F, R>(T, Mc, acc);
}

// contract<2, 1> written with dot products instead of the order-3 tensor:
// with the source's quadratic form q(R) = sum_{|s|=2} Mc_s R^s, its gradient
// v = grad q, d = sum_{|s|=1} Mc_s R^s and tr = Mc_xx + Mc_yy + Mc_zz,
//     sum_s Mc_s T_s       = Mc_0 g_0 + (d + tr) g_1 + q g_2
//     sum_s Mc_s T_{s+e_a} = R_a (Mc_0 g_1 + (d + tr) g_2 + q g_3)
//                            + Mc_{e_a} g_1 + v_a g_2
// (T_{s+e_a} = d/dR_a T_s and d/dR_a g_j = R_a g_{j+1}).  About 35 operations
// instead of the 75 of the tensor recursion and the full contraction.  tr is
// supplied by the caller (stored with the source); AMOEBA has g_0 = 0.
template <typename R>
__host__ __device__ __forceinline__ void contract_q1(R X, R Y, R Z, const R* g, const R* Mc, R tr, int damp,
                                                     R* acc) {
    const R X2 = X + X, Y2 = Y + Y, Z2 = Z + Z;
    const R vx = Mc[4] * X2 + Mc[5] * Y + Mc[6] * Z;
    const R vy = Mc[5] * X + Mc[7] * Y2 + Mc[8] * Z;
    const R vz = Mc[6] * X + Mc[8] * Y + Mc[9] * Z2;
    const R q = (R)0.5 * (X * vx + Y * vy + Z * vz);
    const R dtr = Mc[1] * X + Mc[2] * Y + Mc[3] * Z + tr;
    const R sc = Mc[0] * g[1] + dtr * g[2] + q * g[3];
    R a0 = dtr * g[1] + q * g[2];
    if (damp != DAMP_AMOEBA) a0 += Mc[0] * g[0];
    acc[0] += a0;
    acc[1] += X * sc + Mc[1] * g[1] + vx * g[2];
    acc[2] += Y * sc + Mc[2] * g[1] + vy * g[2];
    acc[3] += Z * sc + Mc[3] * g[1] + vz * g[2];
}

// FP32 pair with an accurate displacement: r^2 is formed with FMA-captured
// rounding errors and 1/r refined by one Newton step on the compensated r^2,
// so 1/r carries about one rounding instead of rsqrtf's few.
// For M = 2, F = 1, Mc[10] holds the trace Mc_xx + Mc_yy + Mc_zz.
template <int M, int F>
__device__ __forceinline__ void pair_field_f32acc(float dx, float dy, float dz, float a, int damp, const float* Mc,
                                                  float* acc) {
    constexpr int N = M + F;
    const float px = dx * dx, py = dy * dy, pz = dz * dz;
    const float ex = fmaf(dx, dx, -px), ey = fmaf(dy, dy, -py), ez = fmaf(dz, dz, -pz);
    const float s1 = px + py;
    const float e1 = (px - (s1 - (s1 - px))) + (py - (s1 - px));  // two-sum error of px + py
    const float r2 = s1 + pz;
    const float e2 = (s1 - (r2 - (r2 - s1))) + (pz - (r2 - s1));
    const float r2lo = (ex + ey + ez) + (e1 + e2);
    const float y0 = rsqrtf(r2);
    const float h = r2 * y0;
    const float hl = fmaf(r2, y0, -h);
    const float res = fmaf(-h, y0, 1.0f) - (hl + r2lo * y0) * y0;
    const float c = 0.5f * y0 * res;
    const float ir = y0 + c;
    const float ir_lo = c - (ir - y0);  // exact: |c| << y0
    float g[N + 1];
    radial_g_ir<N, float>(damp, r2, ir, a, g, ir_lo * (r2 * ir));
    if constexpr (M == 2 && F == 1) {
        contract_q1<float>(dx, dy, dz, g, Mc, Mc[10], damp, acc);
    } else {
        float T[nT(N)];
        md_tensor<N, float>(dx, dy, dz, g, T);
        contract<M, F, float>(T, Mc, acc);
    }
}

// Out-of-line variant for cold paths (exclusion fix-ups) to keep code size down.
template <int M, int F, typename R>
__device__ __noinline__ void pair_field_cold(R dx, R dy, R dz, R a, int damp, const R* Mc, R* acc) {
    pair_field<M, F, R>(dx, dy, dz, a, damp, Mc, acc);
}

}  // namespace fmm

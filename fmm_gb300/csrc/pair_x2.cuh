// Packed FP32 pair arithmetic for the near field: two source particles per
// thread in one 64-bit register pair.
//
// Blackwell executes add, sub, mul and fma on two FP32 values with one
// instruction (`add/sub/mul/fma.rn.f32x2`) at the FMA pipe's element rate of
// the scalar forms, so packing halves the issue slots the arithmetic takes;
// the one-source near field was bound by instruction issue, not by the FMA
// pipe, so a target is evaluated against two sources at once.  Each half
// rounds exactly as the scalar FP32 instruction would (round to nearest,
// IEEE denormals), so a packed pair equals the scalar evaluation written with
// the same operation order.  The transcendental pieces (rsqrt, exp) and the
// rare in-range damping tables run per half.
#pragma once

#include "pair.cuh"

namespace fmm {

struct f2 {
    unsigned long long v;
};

__device__ __forceinline__ f2 mk2(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ f2 bc2(float a) { return mk2(a, a); }
__device__ __forceinline__ void sp2(f2 x, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v)); }
__device__ __forceinline__ float lo2(f2 x) {
    float a, b;
    sp2(x, a, b);
    return a;
}
__device__ __forceinline__ float hi2(f2 x) {
    float a, b;
    sp2(x, a, b);
    return b;
}
__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 operator-(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
// a * b + c, one rounding per half
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return d;
}
__device__ __forceinline__ f2 operator*(float a, f2 b) { return bc2(a) * b; }
__device__ __forceinline__ f2& operator+=(f2& a, f2 b) { return a = a + b; }

// Damped or undamped radial functions g_0..g_N of two pairs (as radial_g_ir
// per half).  Both halves beyond the interval tables (the common case in the
// near field) take the packed closed forms; otherwise each half runs the
// scalar routine.
// CORR: the damped kernel's difference from the undamped one (g_damped -
// g_undamped, AMOEBA only): the closed form keeps just its exponential part,
// so the difference carries no cancellation.
template <int N, bool CORR = false>
__device__ __forceinline__ void radial_g_x2(int damp, f2 r2, f2 ir, f2 a, f2 eps, f2* g) {
    const f2 ir2 = ir * ir;
    f2 num[N + 1];
    bool packed = true;
    if (damp == DAMP_NONE) {
#pragma unroll
        for (int j = 0; j <= N; ++j) num[j] = bc2((float)((j % 2 ? -1.0 : 1.0) * dfact_odd(j)));
    } else if (damp == DAMP_AMOEBA) {
        const f2 x = a * (r2 * ir);
        const f2 u = x * x * x;
        float u0, u1;
        sp2(u, u0, u1);
        packed = !(u0 < Real<float>::kAmoebaHi) && !(u1 < Real<float>::kAmoebaHi);
        if (packed) {
            const f2 e = mk2(Real<float>::expc_(-u0), Real<float>::expc_(-u1));
            num[0] = bc2(CORR ? -1.0f : 0.0f);
#pragma unroll
            for (int j = 1; j <= N; ++j) {
                f2 q = bc2(Real<float>::amoebaQ(j, j - 1));
#pragma unroll
                for (int d = j - 2; d >= 0; --d) q = fma2(q, u, bc2(Real<float>::amoebaQ(j, d)));
                num[j] = CORR ? e * q : fma2(e, q, bc2((float)((j % 2 ? -1.0 : 1.0) * dfact_odd(j))));
            }
        }
    } else if (damp == DAMP_THOLE) {
        const f2 x = a * (r2 * ir);
        float x0, x1;
        sp2(x, x0, x1);
        packed = !(x0 < Real<float>::kTholeHi) && !(x1 < Real<float>::kTholeHi);
        if (packed) {
            const f2 e = mk2(Real<float>::expc_(-x0), Real<float>::expc_(-x1));
            const f2 x2 = x * x;
            const f2 hx2 = bc2(0.5f) * x2;
            f2 ym1 = bc2(1.0f), y0 = bc2(-1.0f) - x;  // Yukawa numerators y_0, y_1
            num[0] = bc2(1.0f) - e * fma2(bc2(0.5f), x, bc2(1.0f));
#pragma unroll
            for (int j = 1; j <= N; ++j) {
                const f2 P = y0 - hx2 * ym1;
                num[j] = bc2((float)((j % 2 ? -1.0 : 1.0) * dfact_odd(j))) - e * P;
                const f2 yn = x2 * ym1 - bc2((float)(2 * j + 1)) * y0;
                ym1 = y0;
                y0 = yn;
            }
        }
    } else {
        packed = false;
    }
    if (packed) {
        f2 irp = ir;
#pragma unroll
        for (int j = 0; j <= N; ++j) {
            const f2 v = num[j] * irp;
            g[j] = fma2(v, bc2((float)(2 * j + 1)) * eps, v);
            irp = irp * ir2;
        }
        return;
    }
    // per half, scalar
    float gh[2][N + 1];
    float r2h[2], irh[2], ah[2], eh[2];
    sp2(r2, r2h[0], r2h[1]);
    sp2(ir, irh[0], irh[1]);
    sp2(a, ah[0], ah[1]);
    sp2(eps, eh[0], eh[1]);
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        radial_g_ir<N, float>(damp, r2h[h], irh[h], ah[h], gh[h], eh[h]);
        if (CORR) {
            // inside the tables the difference is of the order of the terms
            float gu[N + 1];
            radial_g_ir<N, float>(DAMP_NONE, r2h[h], irh[h], ah[h], gu, eh[h]);
#pragma unroll
            for (int j = 0; j <= N; ++j) gh[h][j] -= gu[j];
        }
    }
#pragma unroll
    for (int j = 0; j <= N; ++j) g[j] = mk2(gh[0][j], gh[1][j]);
}

// contract_q1 (quadrupole sources, field order 1) on two pairs, with the
// off-diagonal second moments Mc_xy, Mc_xz, Mc_yz supplied halved: then
// w = grad q / 2 = (Mc_xx X + Mc_xy/2 Y + Mc_xz/2 Z, ...), q = R . w, and the
// gradient term v g_2 of contract_q1 is w (2 g_2).
__device__ __forceinline__ void contract_q1_x2(f2 X, f2 Y, f2 Z, const f2* g, const f2* Mc, int damp, f2* acc) {
    const f2 wx = fma2(Mc[4], X, fma2(Mc[5], Y, Mc[6] * Z));
    const f2 wy = fma2(Mc[5], X, fma2(Mc[7], Y, Mc[8] * Z));
    const f2 wz = fma2(Mc[6], X, fma2(Mc[8], Y, Mc[9] * Z));
    const f2 q = fma2(X, wx, fma2(Y, wy, Z * wz));
    const f2 dtr = fma2(Mc[1], X, fma2(Mc[2], Y, fma2(Mc[3], Z, Mc[10])));
    const f2 sc = fma2(Mc[0], g[1], fma2(dtr, g[2], q * g[3]));
    const f2 g2d = g[2] + g[2];
    f2 a0 = fma2(dtr, g[1], q * g[2]);
    if (damp != DAMP_AMOEBA) a0 = fma2(Mc[0], g[0], a0);
    acc[0] += a0;
    acc[1] += fma2(X, sc, fma2(Mc[1], g[1], wx * g2d));
    acc[2] += fma2(Y, sc, fma2(Mc[2], g[1], wy * g2d));
    acc[3] += fma2(Z, sc, fma2(Mc[3], g[1], wz * g2d));
}

// Cartesian derivative tensor of all orders <= N (md_tensor) on two pairs.
template <int N>
__device__ __forceinline__ void md_tensor_x2(f2 X, f2 Y, f2 Z, const f2* g, f2* T) {
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
                    f2 v;
                    if (tx > 0) {
                        v = X * T[pidx(tx - 1, ty, tz)];
                        if (tx > 1) v = fma2(bc2((float)(tx - 1)), T[pidx(tx - 2, ty, tz)], v);
                    } else if (ty > 0) {
                        v = Y * T[pidx(tx, ty - 1, tz)];
                        if (ty > 1) v = fma2(bc2((float)(ty - 1)), T[pidx(tx, ty - 2, tz)], v);
                    } else {
                        v = Z * T[pidx(tx, ty, tz - 1)];
                        if (tz > 1) v = fma2(bc2((float)(tz - 1)), T[pidx(tx, ty, tz - 2)], v);
                    }
                    T[pidx(tx, ty, tz)] = v;
                }
            }
        }
        T[0] = g[j];
    }
}

template <int M, int F>
__device__ __forceinline__ void contract_x2(const f2* T, const f2* Mc, f2* acc) {
#pragma unroll
    for (int fo = 0; fo <= F; ++fo)
#pragma unroll
        for (int fx = fo; fx >= 0; --fx)
#pragma unroll
            for (int fy = fo - fx; fy >= 0; --fy) {
                const int fz = fo - fx - fy;
                f2 a = acc[pidx(fx, fy, fz)];
#pragma unroll
                for (int so = 0; so <= M; ++so)
#pragma unroll
                    for (int sx = so; sx >= 0; --sx)
#pragma unroll
                        for (int sy = so - sx; sy >= 0; --sy) {
                            const int sz = so - sx - sy;
                            a = fma2(Mc[pidx(sx, sy, sz)], T[pidx(sx + fx, sy + fy, sz + fz)], a);
                        }
                acc[pidx(fx, fy, fz)] = a;
            }
}

// pair_field_f32acc on two pairs: compensated r^2 (FMA-captured product
// errors, TwoSum of the squares), one Newton step for 1/r on the compensated
// r^2, radial functions with the 1/r correction, contraction.
// CORR: the damping correction of a pair (AMOEBA): the field of the damped
// kernel minus that of the undamped one, potential term included.
template <int M, int F, bool CORR = false>
__device__ __forceinline__ void pair_field_x2(f2 dx, f2 dy, f2 dz, f2 a, int damp, const f2* Mc, f2* acc) {
    constexpr int N = M + F;
    const f2 px = dx * dx, py = dy * dy, pz = dz * dz;
    const f2 ndx = bc2(0.0f) - dx, ndy = bc2(0.0f) - dy, ndz = bc2(0.0f) - dz;
    // -(exact square - rounded square), per axis
    const f2 nex = fma2(ndx, dx, px), ney = fma2(ndy, dy, py), nez = fma2(ndz, dz, pz);
    const f2 s1 = px + py;
    const f2 t1 = s1 - px;
    const f2 e1 = (px - (s1 - t1)) + (py - t1);
    const f2 r2 = s1 + pz;
    const f2 t2 = r2 - s1;
    const f2 e2 = (s1 - (r2 - t2)) + (pz - t2);
    const f2 r2lo = (e1 + e2) - (nex + ney + nez);
    float ra, rb;
    sp2(r2, ra, rb);
    const f2 y0 = mk2(rsqrtf(ra), rsqrtf(rb));
    const f2 h = r2 * y0;
    const f2 nh = bc2(0.0f) - h;
    const f2 hl = fma2(r2, y0, nh);
    const f2 res = fma2(nh, y0, bc2(1.0f)) - fma2(r2lo, y0, hl) * y0;
    const f2 c = bc2(0.5f) * y0 * res;
    const f2 ir = y0 + c;
    const f2 ir_lo = c - (ir - y0);
    f2 g[N + 1];
    radial_g_x2<N, CORR>(damp, r2, ir, a, ir_lo * (r2 * ir), g);
    if constexpr (M == 2 && F == 1) {
        contract_q1_x2(dx, dy, dz, g, Mc, CORR ? (int)DAMP_NONE : damp, acc);
    } else {
        f2 T[nT(N)];
        md_tensor_x2<N>(dx, dy, dz, g, T);
        contract_x2<M, F>(T, Mc, acc);
    }
}

}  // namespace fmm

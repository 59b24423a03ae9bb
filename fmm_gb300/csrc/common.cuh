// Shared definitions of the GB300 fmm field-evaluation library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fmm_gpu.h"

namespace fmm {

enum Damp : int { DAMP_NONE = 0, DAMP_AMOEBA = 1, DAMP_THOLE = 2, DAMP_ERF = 3 };

constexpr int kMaxP = 12;       // highest expansion order built
constexpr int kMaxDepth = 21;   // octree levels that fit a 63-bit key (3 bits per level)
constexpr int kWarp = 32;

// Number of packed components of all orders <= k: (k+1)(k+2)(k+3)/6.
__host__ __device__ constexpr int nT(int k) { return k < 0 ? 0 : (k + 1) * (k + 2) * (k + 3) / 6; }

// Packed alphabetical index (0-based) of the component x^a y^b z^c.  Within
// order k the components run with the x power descending, then the y power
// descending: xx, xy, xz, yy, yz, zz (src/fmm.F90:80-89 xyz2idx, 1-based there).
__host__ __device__ constexpr int pidx(int x, int y, int z) {
    return nT(x + y + z - 1) + ((y + z) * (y + z + 1)) / 2 + z;
}

// Inverse of pidx, usable in constant expressions.
__host__ __device__ constexpr int order_of(int q) {
    int k = 0;
    while (nT(k) <= q) ++k;
    return k;
}
__host__ __device__ constexpr int comp_w(int q) {  // y + z
    int l = q - nT(order_of(q) - 1);
    int w = 0;
    while ((w + 1) * (w + 2) / 2 <= l) ++w;
    return w;
}
__host__ __device__ constexpr int comp_z(int q) { return q - nT(order_of(q) - 1) - comp_w(q) * (comp_w(q) + 1) / 2; }
__host__ __device__ constexpr int comp_y(int q) { return comp_w(q) - comp_z(q); }
__host__ __device__ constexpr int comp_x(int q) { return order_of(q) - comp_w(q); }

// Packed index of component(s) + component(f).
__host__ __device__ constexpr int sum_idx(int s, int f) {
    return pidx(comp_x(s) + comp_x(f), comp_y(s) + comp_y(f), comp_z(s) + comp_z(f));
}

__host__ __device__ constexpr double cfact(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= (double)i;
    return f;
}

// Index of the first packed component of order k.
__host__ __device__ constexpr int order_start(int k) { return nT(k - 1); }

inline int dim_to_order(int dim) {
    for (int m = 0; m <= 16; ++m)
        if (nT(m) == dim) return m;
    return -1;
}

#ifdef __CUDACC__
// NORM2 of a 3-vector as the scaled sum of squares gfortran expands it to,
// in a fixed sequence of correctly rounded operations (the reference's tie
// decisions depend on its last bit, src/fmm.F90:358-364).
__device__ __forceinline__ double norm2_3(double a0, double a1, double a2) {
    double scale = 0.0, ssq = 1.0;
    const double v[3] = {a0, a1, a2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (v[i] != 0.0) {
            const double ax = fabs(v[i]);
            if (scale < ax) {
                const double t = __ddiv_rn(scale, ax);
                ssq = __dadd_rn(1.0, __dmul_rn(__dmul_rn(ssq, t), t));
                scale = ax;
            } else {
                const double t = __ddiv_rn(ax, scale);
                ssq = __dadd_rn(ssq, __dmul_rn(t, t));
            }
        }
    }
    return __dmul_rn(scale, __dsqrt_rn(ssq));
}
#endif

#define FMM_CUDA_TRY(expr)                         \
    do {                                           \
        cudaError_t e_ = (expr);                   \
        if (e_ != cudaSuccess) return FMM_ECUDA;   \
    } while (0)

#define FMM_TRY(expr)              \
    do {                           \
        int s_ = (expr);           \
        if (s_ != FMM_OK) return s_; \
    } while (0)

}  // namespace fmm

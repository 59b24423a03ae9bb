// Index maps of the harmonic reduced basis used by the exact-coefficient M2L.
//
// Restricted tensor: the Cartesian derivatives T_(t,u,v) of 1/r with z-index
// v <= 2, ordered by total order n, then v, then u (2n+1 + n entries per
// order, all that a reduced-basis contraction reads).
// Reduced basis: the (k+1)^2 components (x, y, z) with z <= 1 of all orders
// <= k; order k's block of 2k+1 entries starts at k^2, z = 0 first.
#pragma once

#include "common.cuh"

namespace fmm {

__host__ __device__ constexpr int rbase(int n) { return n == 0 ? 0 : 1 + 3 * (n - 1) * n / 2; }
__host__ __device__ constexpr int ridx(int t, int u, int v) {
    const int n = t + u + v;
    return rbase(n) + (v == 0 ? 0 : (v == 1 ? n + 1 : 2 * n + 1)) + u;
}
__host__ __device__ constexpr int qidx(int x, int y, int z) {
    const int k = x + y + z;
    return k * k + (z == 0 ? y : k + 1 + y);
}

// Reduced index q -> packed (x, y, z, k) = x | y << 8 | z << 16 | k << 24.
__host__ __device__ __forceinline__ int qcomp(int q) {
    int k = 0;
    while ((k + 1) * (k + 1) <= q) ++k;
    const int l = q - k * k;
    const int z = l <= k ? 0 : 1;
    const int y = z == 0 ? l : l - (k + 1);
    const int x = k - y - z;
    return x | (y << 8) | (z << 16) | (k << 24);
}

// Recursion rule of restricted entry e: the Hermite step along the first axis
// with a positive index, R_e = X_dir R'_par + cnt R'_gp (primes: one level
// up).  Packed as (par | dir << 16, gp | cnt << 16).
__host__ __device__ __forceinline__ int2 restricted_rule(int e) {
    int n = 0;
    while (rbase(n + 1) <= e) ++n;
    const int l = e - rbase(n);
    const int v = l <= n ? 0 : (l <= 2 * n ? 1 : 2);
    const int u = l - (v == 0 ? 0 : (v == 1 ? n + 1 : 2 * n + 1));
    const int tt = n - v - u;
    int dir = 0, par = 0, gp = 0, cnt = 0;
    if (tt > 0) {
        dir = 0; par = ridx(tt - 1, u, v); cnt = tt - 1; gp = tt > 1 ? ridx(tt - 2, u, v) : 0;
    } else if (u > 0) {
        dir = 1; par = ridx(0, u - 1, v); cnt = u - 1; gp = u > 1 ? ridx(0, u - 2, v) : 0;
    } else if (v > 0) {
        dir = 2; par = ridx(0, 0, v - 1); cnt = v - 1; gp = v > 1 ? ridx(0, 0, v - 2) : 0;
    }
    return make_int2(par | (dir << 16), gp | (cnt << 16));
}

}  // namespace fmm

// CPU oracle for the fmm field-evaluation path.
//
// TEST INFRASTRUCTURE ONLY.  This file is a plain C++ restatement of the
// reference library's `field_direct` / `field_fmm` (peter-reinholdt/fmm,
// src/fmm.F90) and of its interaction tensors (src/tensors_recursive.F90,
// src/tensors_damped_{amoeba,thole,erf}.F90).  Only the tests, the smoke
// check and the CPU-baseline leg of the benchmark load it, and only as the
// checker.  The product library (fmm_gb300) never links or calls it.
//
// Parity status: pinned to the reference's own code.  The reference is
// Fortran, has no tests or fixtures, and no Fortran compiler exists here; its
// source statements are instead executed through a mechanical translation
// (tests/golden/fortran_exec.py) that writes golden fixtures
// (tests/golden/ref_*.npz).  tests/test_ref_golden.py checks this file against
// them: the int32 Cnij table and the octree and interaction lists bit for bit,
// Tn_recursive (orders <= 16), the generated T0..T12 and the damped T0..T6 of
// all three kinds to 1e-13, and field_direct / field_fmm of five systems
// (every damping kind, multipole orders 0-2, field orders 1-2, expansion
// orders 4-8) to 1e-12 relative.
//
// Two families of behaviour are selectable per call (OracleOpts):
//   coef_mode  0 = "ref":   undamped tensors by the reference's closed form
//                           (tensors_recursive.F90:29-135) with the Cnij
//                           table in two's-complement int32, as the default
//                           gfortran build computes it (it wraps for tensor
//                           order >= 11); damped tensors truncated above
//                           order 6 like tensors_damped_*.F90:57-63.
//              1 = "exact": Cnij in 128-bit integers (order <= 16 is exact,
//                           as a -DINT64 build would be), damped tensors at
//                           every order.
//   excl_mode  0 = "ref1e10": excluded sources are moved to R=(1e10,1e10,1e10)
//                           (fmm.F90:714-720, 802-806); the self pair is only
//                           skipped if it is listed.
//              1 = "mask":  excluded pairs and the self pair are skipped; in
//                           field_fmm, excluded pairs that fall in the far
//                           field are subtracted again (their undamped pair
//                           field), which the reference never does
//                           (fmm.F90:861-877 has no exclusion handling).
//   centroid_mode 0 = sequential sum of the coordinates (fmm.F90:184, the
//                           order gfortran's SUM uses), 1 = the blocked sum
//                           the GPU build uses (lane l of 1024 sums elements
//                           l, l+1024, ... in order, then the 1024 lane sums
//                           are added in lane order).
//
// All floating-point expressions follow the reference's evaluation order
// where that is cheap to do; the file is compiled with -ffp-contract=off.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
struct OracleOpts {
    int coef_mode;      // 0 ref, 1 exact
    int excl_mode;      // 0 ref1e10, 1 mask
    int centroid_mode;  // 0 sequential, 1 blocked(1024 lanes)
    int nthreads;       // <=0: library default
    int mac_mode;       // 0 reference MAC, 1 also demote pairs within the damping range
    double target_rel_err;
};
}

namespace {

enum { DAMP_NONE = 0, DAMP_AMOEBA = 1, DAMP_THOLE = 2, DAMP_ERF = 3 };
enum { OK = 0, E_INVAL = -1, E_NOTSUP = -2, E_DEPTH = -5 };

inline int nT(int k) { return (k + 1) * (k + 2) * (k + 3) / 6; }
// order of the packed component c (nT(order - 1) <= c < nT(order))
inline int order_of(int c) {
    int k = 0;
    while (nT(k) <= c) ++k;
    return k;
}

// Packed alphabetical index, 0-based (fmm.F90:80-89 xyz2idx, which is 1-based).
inline int pidx(int x, int y, int z) {
    int k = x + y + z;
    return k * (k + 1) * (k + 2) / 6 + (y * y + 2 * y * z + y + z * z + 3 * z) / 2;
}

// fmm.F90:91-111
double factorial(int n) {
    double f = 1.0;
    for (int i = n; i >= 1; --i) f = f * (double)i;
    return f;
}
double binom(int n, int k) { return factorial(n) / (factorial(k) * factorial(n - k)); }
double trinom(int i, int j, int k) { return factorial(i + j + k) / ((factorial(i) * factorial(j)) * factorial(k)); }

// real**integer as gfortran lowers it for a non-constant exponent: binary
// exponentiation, squaring the base and multiplying right to left.
double ipow(double x, int m) {
    unsigned n = (unsigned)m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) {
        x = x * x;
        if (n % 2) y = y * x;
    }
    return y;
}

// NORM2 of a 3-vector with the scaled sum of squares gfortran expands it to.
double norm2_3(double a0, double a1, double a2) {
    double scale = 0.0, ssq = 1.0;
    const double v[3] = {a0, a1, a2};
    for (int i = 0; i < 3; ++i) {
        if (v[i] != 0.0) {
            double ax = std::fabs(v[i]);
            if (scale < ax) {
                double t = scale / ax;
                ssq = 1.0 + (ssq * t) * t;
                scale = ax;
            } else {
                double t = ax / scale;
                ssq = ssq + t * t;
            }
        }
    }
    return scale * std::sqrt(ssq);
}

int dim_to_order(int dim) {
    for (int m = 0; m < 16; ++m)
        if (nT(m) == dim) return m;
    return -1;
}

// ---------------------------------------------------------------------------
// Cnij coefficient table (tensors_recursive.F90:64-93).
struct Cnij {
    int maxo = -1;
    int d0 = 0, d1 = 0;  // extents: n in [1, 2*maxo+3], i,j in [0, maxo+1]
    std::vector<double> v;
    double get(int n, int i, int j) const { return v[((size_t)(n - 1) * d1 + i) * d1 + j]; }
};

Cnij make_cnij(int maxo, bool wrap32) {
    Cnij t;
    t.maxo = maxo;
    t.d0 = 2 * maxo + 3;
    t.d1 = maxo + 2;
    std::vector<__int128> e((size_t)t.d0 * t.d1 * t.d1, 0);
    std::vector<int32_t> w((size_t)t.d0 * t.d1 * t.d1, 0);
    auto at = [&](int n, int i, int j) { return ((size_t)(n - 1) * t.d1 + i) * t.d1 + j; };
    for (int n = 1; n <= t.d0; ++n) {
        e[at(n, 0, 0)] = 1;
        w[at(n, 0, 0)] = 1;
    }
    for (int n = 1; n <= t.d0; ++n) {
        if (n % 2 == 0) continue;
        for (int i = 1; i <= maxo + 1; ++i) {
            int k = (i % 2 != 0) ? i - 1 : i;
            for (int j = 0; j <= i; ++j) {
                if ((i + j) % 2 != 0) continue;
                if (j == 0) {
                    e[at(n, i, j)] = e[at(n, i - 1, j + 1)];
                    w[at(n, i, j)] = w[at(n, i - 1, j + 1)];
                } else if (j != i) {
                    e[at(n, i, j)] = (__int128)(j + 1) * e[at(n, i - 1, j + 1)] - (__int128)(n + k) * e[at(n, i - 1, j - 1)];
                    uint32_t a = (uint32_t)(j + 1) * (uint32_t)w[at(n, i - 1, j + 1)];
                    uint32_t b = (uint32_t)(n + k) * (uint32_t)w[at(n, i - 1, j - 1)];
                    w[at(n, i, j)] = (int32_t)(a - b);
                    k = k + 2;
                } else {
                    e[at(n, i, j)] = -(__int128)(n + k) * e[at(n, i - 1, j - 1)];
                    w[at(n, i, j)] = (int32_t)((uint32_t)0 - (uint32_t)(n + k) * (uint32_t)w[at(n, i - 1, j - 1)]);
                }
            }
        }
    }
    t.v.resize(e.size());
    for (size_t q = 0; q < e.size(); ++q) t.v[q] = wrap32 ? (double)w[q] : (double)e[q];
    return t;
}

// Undamped T tensors by the closed form (tensors_recursive.F90:29-62, 95-135).
// T is column-major (ns, nT(nmax)).
void tn_closed(int nmax, int ns, const double* x, const double* y, const double* z, double* T, const Cnij& C) {
    std::vector<double> xp((size_t)(nmax + 1)), yp((size_t)(nmax + 1)), zp((size_t)(nmax + 1));
    for (int s = 0; s < ns; ++s) {
        double R = std::sqrt((x[s] * x[s] + y[s] * y[s]) + z[s] * z[s]);
        xp[0] = yp[0] = zp[0] = 1.0;
        for (int i = 1; i <= nmax; ++i) {
            xp[i] = xp[i - 1] * (x[s] / R);
            yp[i] = yp[i - 1] * (y[s] / R);
            zp[i] = zp[i - 1] * (z[s] / R);
        }
        int idx = 0;
        for (int n = 0; n <= nmax; ++n) {
            double invR = 1.0 / ipow(R, n + 1);
            for (int kx = n; kx >= 0; --kx)
                for (int ky = n - kx; ky >= 0; --ky) {
                    int kz = n - kx - ky;
                    double acc = 0.0;
                    for (int a = 0; a <= kx; ++a) {
                        double c1 = C.get(1, kx, a);
                        if (c1 == 0.0) continue;
                        double Cx = c1 * xp[a];
                        for (int b = 0; b <= ky; ++b) {
                            double c2 = C.get(a + kx + 1, ky, b);
                            if (c2 == 0.0) continue;
                            double Cy = (Cx * c2) * yp[b];
                            for (int c = 0; c <= kz; ++c) {
                                double c3 = C.get(a + kx + b + ky + 1, kz, c);
                                if (c3 == 0.0) continue;
                                acc = acc + (Cy * c3) * zp[c];
                            }
                        }
                    }
                    T[(size_t)idx * ns + s] = acc * invR;
                    ++idx;
                }
        }
    }
}

// ---------------------------------------------------------------------------
// Radial derivative functions g_j(r) = (r^-1 d/dr)^j phi(r), j = 0..n, for
// the damped kernels of tensors_damped_*.F90:
//   THOLE : phi = (1 - (1 + a r/2) e^{-a r}) / r
//   ERF   : phi = erf(sqrt(a) r) / r
//   AMOEBA: g_1 = -(1 - e^{-a^3 r^3}) / r^3, g_0 := 0 (T0 is identically 0)
// Small arguments use power series (term-wise derivative of the Taylor
// series in r); large arguments use closed forms / upward recursions.

// product m (m-2) (m-4) ... (m-2j+2): (r^-1 d/dr)^j r^m = P r^(m-2j)
double power_rule(int m, int j) {
    double p = 1.0;
    for (int i = 0; i < j; ++i) p *= (double)(m - 2 * i);
    return p;
}

double dfact_odd(int j) {  // (2j-1)!!, with (-1)!! = 1
    double p = 1.0;
    for (int i = 1; i <= j; ++i) p *= (double)(2 * i - 1);
    return p;
}

void radial_g(int damp, double r, double a, int n, double* g) {
    if (damp == DAMP_NONE) {
        double ir2 = 1.0 / (r * r);
        g[0] = 1.0 / r;
        for (int j = 1; j <= n; ++j) g[j] = -(double)(2 * j - 1) * g[j - 1] * ir2;
        return;
    }
    if (damp == DAMP_THOLE) {
        double x = a * r;
        if (x < 1.0) {
            // phi = sum_{k>=1} c_k a^k r^(k-1), c_k = (-1)^(k+1) (1 - k/2) / k!
            for (int j = 0; j <= n; ++j) g[j] = 0.0;
            double ak = 1.0, kf = 1.0;
            for (int k = 1; k <= 40; ++k) {
                ak *= a;
                kf *= (double)k;
                double ck = ((k % 2) ? 1.0 : -1.0) * (1.0 - 0.5 * k) / kf;
                if (ck == 0.0) continue;
                for (int j = 0; j <= n; ++j) {
                    double pr = power_rule(k - 1, j);
                    if (pr == 0.0) continue;
                    g[j] += ck * ak * pr * std::pow(r, (double)(k - 1 - 2 * j));
                }
            }
            return;
        }
        double e = std::exp(-x);
        std::vector<double> yv((size_t)n + 2);
        yv[0] = 1.0;
        yv[1] = -(1.0 + x);
        for (int j = 1; j <= n; ++j) yv[j + 1] = x * x * yv[j - 1] - (double)(2 * j + 1) * yv[j];
        double rp = r;
        for (int j = 0; j <= n; ++j) {
            double P = (j == 0) ? (1.0 + 0.5 * x) : (yv[j] - 0.5 * x * x * yv[j - 1]);
            double sgn = (j % 2) ? -1.0 : 1.0;
            g[j] = (sgn * dfact_odd(j) - e * P) / rp;
            rp *= r * r;
        }
        return;
    }
    if (damp == DAMP_ERF) {
        double beta = std::sqrt(a);
        double s = a * r * r;
        std::vector<double> F((size_t)n + 1);
        double es = std::exp(-s);
        if (s < 30.0) {
            // F_n(s) = e^{-s} sum_k (2s)^k / ((2n+1)(2n+3)...(2n+2k+1)), then downward
            double term = 1.0 / (2.0 * n + 1.0), sum = term;
            for (int k = 1; k < 400; ++k) {
                term *= 2.0 * s / (2.0 * n + 2.0 * k + 1.0);
                sum += term;
                if (term < 1e-20 * sum) break;
            }
            F[n] = es * sum;
            for (int j = n - 1; j >= 0; --j) F[j] = (2.0 * s * F[j + 1] + es) / (2.0 * j + 1.0);
        } else {
            double rs = std::sqrt(s);
            F[0] = 0.5 * std::sqrt(M_PI) * std::erf(rs) / rs;
            for (int j = 0; j < n; ++j) F[j + 1] = ((2.0 * j + 1.0) * F[j] - es) / (2.0 * s);
        }
        double pre = beta * 2.0 / std::sqrt(M_PI);
        for (int j = 0; j <= n; ++j) {
            g[j] = ((j % 2) ? -1.0 : 1.0) * pre * F[j];
            pre *= 2.0 * beta * beta;
        }
        return;
    }
    // AMOEBA
    g[0] = 0.0;
    if (n == 0) return;
    double x = a * r;
    if (x < 1.0) {
        // g_1 = -sum_{k>=1} (-1)^(k+1) a^(3k) r^(3k-3) / k!
        for (int j = 1; j <= n; ++j) g[j] = 0.0;
        double a3k = 1.0, kf = 1.0;
        for (int k = 1; k <= 30; ++k) {
            a3k *= a * a * a;
            kf *= (double)k;
            double ck = -((k % 2) ? 1.0 : -1.0) / kf;
            for (int j = 1; j <= n; ++j) {
                double pr = power_rule(3 * k - 3, j - 1);
                if (pr == 0.0) continue;
                g[j] += ck * a3k * pr * std::pow(r, (double)(3 * k - 3 - 2 * (j - 1)));
            }
        }
        return;
    }
    double u = x * x * x;
    double e = std::exp(-u);
    // Q_1 = 1, Q_{j+1}(u) = 3u (Q_j' - Q_j) - (2j+1) Q_j
    std::vector<double> Q(1, 1.0);
    double rp = r * r * r;
    for (int j = 1; j <= n; ++j) {
        double qv = 0.0;
        for (int d = (int)Q.size() - 1; d >= 0; --d) qv = qv * u + Q[d];
        double sgn = (j % 2) ? -1.0 : 1.0;
        g[j] = (sgn * dfact_odd(j) + e * qv) / rp;
        rp *= r * r;
        std::vector<double> Qn(Q.size() + 1, 0.0);
        for (size_t d = 0; d < Q.size(); ++d) {
            Qn[d] -= (double)(2 * j + 1) * Q[d];
            Qn[d + 1] -= 3.0 * Q[d];
            if (d >= 1) Qn[d] += 3.0 * (double)d * Q[d];
        }
        Q.swap(Qn);
    }
}

// Cartesian derivative tensor of the radial function from its g_j by the
// Hermite-type recursion R^(j)_{t+1,u,v} = t R^(j+1)_{t-1,u,v} + X R^(j+1)_{t,u,v}.
void tensor_from_g(int nmax, double X, double Y, double Z, const double* g, double* T /* nT(nmax) */) {
    std::vector<double> cur((size_t)nT(nmax)), nxt((size_t)nT(nmax));
    for (int j = nmax; j >= 0; --j) {
        int lim = nmax - j;
        cur[0] = g[j];
        for (int k = 1; k <= lim; ++k)
            for (int tx = k; tx >= 0; --tx)
                for (int ty = k - tx; ty >= 0; --ty) {
                    int tz = k - tx - ty;
                    double v;
                    if (tx > 0) {
                        v = X * nxt[pidx(tx - 1, ty, tz)];
                        if (tx > 1) v += (double)(tx - 1) * nxt[pidx(tx - 2, ty, tz)];
                    } else if (ty > 0) {
                        v = Y * nxt[pidx(tx, ty - 1, tz)];
                        if (ty > 1) v += (double)(ty - 1) * nxt[pidx(tx, ty - 2, tz)];
                    } else {
                        v = Z * nxt[pidx(tx, ty, tz - 1)];
                        if (tz > 1) v += (double)(tz - 1) * nxt[pidx(tx, ty, tz - 2)];
                    }
                    cur[pidx(tx, ty, tz)] = v;
                }
        std::swap(cur, nxt);
    }
    for (int q = 0; q < nT(nmax); ++q) T[q] = nxt[q];
}

struct Ctx {
    int coef_mode = 0;
    int excl_mode = 0;
    int centroid_mode = 0;
    int mac_mode = 0;
    double target = 1e-6;
    Cnij cn;  // table for the closed-form tensors
    void ensure_cnij(int maxo) {
        if (cn.maxo < maxo) cn = make_cnij(maxo, coef_mode == 0);
    }
};

// All tensors up to order nmax for ns displacements; T column-major (ns, nT(nmax)).
void tensors(int nmax, int ns, const double* x, const double* y, const double* z, int damp, const double* a,
             const Ctx& ctx, double* T) {
    if (damp == DAMP_NONE && ctx.coef_mode == 0) {
        tn_closed(nmax, ns, x, y, z, T, ctx.cn);
        return;
    }
    if (damp == DAMP_NONE && ctx.coef_mode == 1 && nmax <= 16) {
        tn_closed(nmax, ns, x, y, z, T, ctx.cn);
        return;
    }
    std::vector<double> g((size_t)nmax + 1), t((size_t)nT(nmax));
    for (int s = 0; s < ns; ++s) {
        double r = std::sqrt((x[s] * x[s] + y[s] * y[s]) + z[s] * z[s]);
        radial_g(damp, r, damp == DAMP_NONE ? 0.0 : a[s], nmax, g.data());
        tensor_from_g(nmax, x[s], y[s], z[s], g.data(), t.data());
        for (int q = 0; q < nT(nmax); ++q) {
            double v = t[q];
            if (damp != DAMP_NONE && ctx.coef_mode == 0) {
                int ord = 0;
                while (nT(ord) <= q) ++ord;
                if (ord > 6) v = 0.0;
            }
            T[(size_t)q * ns + s] = v;
        }
    }
}

// multipole_field (fmm.F90:548-621): F(nT(pf)) = field at the origin of the
// displacement vectors from ns multipoles M (column-major (ns, dim)).
void multipole_field(int ns, const double* M, int dim, const double* x, const double* y, const double* z, int pf,
                     int damp, const double* a, const Ctx& ctx, double* F, std::vector<double>& Tbuf) {
    int pm = dim_to_order(dim);
    int nmax = pf + pm;
    for (int q = 0; q < nT(pf); ++q) F[q] = 0.0;
    if (ns == 0) return;
    Tbuf.resize((size_t)ns * nT(nmax));
    tensors(nmax, ns, x, y, z, damp, a, ctx, Tbuf.data());
    const double* T = Tbuf.data();
    for (int fo = 0; fo <= pf; ++fo)
        for (int mo = 0; mo <= pm; ++mo) {
            double taylor = ((mo + 1) % 2 ? -1.0 : 1.0) / factorial(mo);
            for (int sx = mo; sx >= 0; --sx)
                for (int sy = mo; sy >= 0; --sy)
                    for (int sz = mo; sz >= 0; --sz) {
                        if (sx + sy + sz != mo) continue;
                        int mi = pidx(sx, sy, sz);
                        for (int tx = fo; tx >= 0; --tx)
                            for (int ty = fo; ty >= 0; --ty)
                                for (int tz = fo; tz >= 0; --tz) {
                                    if (tx + ty + tz != fo) continue;
                                    int fi = pidx(tx, ty, tz);
                                    int ti = pidx(sx + tx, sy + ty, sz + tz);
                                    double symfac = trinom(sx, sy, sz);
                                    double sum = 0.0;
                                    const double* Mc = M + (size_t)mi * ns;
                                    const double* Tc = T + (size_t)ti * ns;
                                    for (int s = 0; s < ns; ++s) sum = sum + Mc[s] * Tc[s];
                                    F[fi] = F[fi] + (taylor * symfac) * sum;
                                }
                    }
        }
}

// ---------------------------------------------------------------------------
// Octree (fmm.F90:137-299): sequential insertion, split on reaching ncrit,
// DFS-preorder numbering.
struct Node {
    int depth = 1;
    int nleaf = 0;
    std::vector<int> leaf;  // 0-based particle indices
    double c[3] = {0, 0, 0};
    double r = 0, rmax = 0;
    int parent = -1;
    int child[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    bool terminal = true;
    int idx = -1;  // DFS id
};

struct Tree {
    std::vector<Node> nd;    // creation order
    std::vector<int> dfs;    // dfs id -> creation index
    int max_depth = 0;
    std::vector<std::vector<int>> far, nearl;  // by dfs id, values are dfs ids
    bool depth_overflow = false;
};

struct Builder {
    const double* X;
    int64_t n;
    int ncrit;
    Tree* t;
    int add_child(int ni, int oct) {
        Node ch;
        Node& pn = t->nd[ni];
        double r = pn.r * 0.5;
        ch.c[0] = pn.c[0] + r * (double)((oct & 1) * 2 - 1);
        ch.c[1] = pn.c[1] + r * (double)((oct & 2) - 1);
        ch.c[2] = pn.c[2] + r * (double)((oct & 4) / 2 - 1);
        ch.r = r;
        ch.rmax = std::sqrt((1.5 * r) * r);
        ch.parent = ni;
        ch.depth = pn.depth + 1;
        if (ch.depth > 64) t->depth_overflow = true;
        t->nd[ni].terminal = false;
        t->nd.push_back(ch);
        int id = (int)t->nd.size() - 1;
        t->nd[ni].child[oct] = id;
        return id;
    }
    int octant(int64_t i, const Node& nd) const {
        int o = 0;
        if (X[i] > nd.c[0]) o += 1;
        if (X[n + i] > nd.c[1]) o += 2;
        if (X[2 * n + i] > nd.c[2]) o += 4;
        return o;
    }
    void split(int ni) {
        if (t->depth_overflow) return;
        std::vector<int> lv = t->nd[ni].leaf;
        int cnt = t->nd[ni].nleaf;
        for (int q = 0; q < cnt; ++q) {
            int p = lv[q];
            int o = octant(p, t->nd[ni]);
            int ci = t->nd[ni].child[o];
            if (ci < 0) ci = add_child(ni, o);
            t->nd[ci].nleaf += 1;
            t->nd[ci].leaf.push_back(p);
            if (t->nd[ci].nleaf >= ncrit) split(ci);
            if (t->depth_overflow) return;
        }
    }
};

void centroid(const double* X, int64_t n, int mode, double c[3]) {
    for (int d = 0; d < 3; ++d) {
        const double* v = X + d * n;
        if (mode == 0) {
            double s = 0.0;
            for (int64_t i = 0; i < n; ++i) s = s + v[i];
            c[d] = s / (double)n;
        } else {
            double lanes[1024];
            for (int l = 0; l < 1024; ++l) {
                double s = 0.0;
                for (int64_t i = l; i < n; i += 1024) s = s + v[i];
                lanes[l] = s;
            }
            double s = 0.0;
            for (int l = 0; l < 1024; ++l) s = s + lanes[l];
            c[d] = s / (double)n;
        }
    }
}

int build_tree(const double* X, int64_t n, int ncrit, int centroid_mode, Tree& t) {
    t.nd.clear();
    t.nd.reserve((size_t)(2 * n / std::max(ncrit, 1) + 16));
    Node root;
    root.depth = 1;
    centroid(X, n, centroid_mode, root.c);
    double m = 0.0;
    for (int d = 0; d < 3; ++d) {
        double md = 0.0;
        for (int64_t i = 0; i < n; ++i) md = std::max(md, std::fabs(X[d * n + i] - root.c[d]));
        m = std::max(m, md);
    }
    root.r = m * 1.0001;
    root.rmax = std::sqrt((1.5 * root.r) * root.r);
    t.nd.push_back(root);
    Builder b{X, n, ncrit, &t};
    for (int64_t i = 0; i < n; ++i) {
        int ni = 0;
        while (t.nd[ni].nleaf >= ncrit) {
            t.nd[ni].nleaf += 1;
            int o = b.octant(i, t.nd[ni]);
            if (t.nd[ni].child[o] < 0) b.add_child(ni, o);
            ni = t.nd[ni].child[o];
        }
        t.nd[ni].nleaf += 1;
        t.nd[ni].leaf.push_back((int)i);
        if (t.nd[ni].nleaf >= ncrit) b.split(ni);
        if (t.depth_overflow) return E_DEPTH;
    }
    // downward_pass: DFS preorder over octants 0..7 (fmm.F90:286-299)
    t.dfs.clear();
    t.max_depth = 0;
    std::vector<int> stack{0};
    while (!stack.empty()) {
        int ni = stack.back();
        stack.pop_back();
        t.nd[ni].idx = (int)t.dfs.size();
        t.dfs.push_back(ni);
        t.max_depth = std::max(t.max_depth, t.nd[ni].depth);
        for (int o = 7; o >= 0; --o)
            if (t.nd[ni].child[o] >= 0) stack.push_back(t.nd[ni].child[o]);
    }
    return OK;
}

// Distance beyond which the damped g_j (j <= nmax) deviate from the undamped
// ones by at most eps (relative): scan of r on a fixed log grid.
double damping_range(int damp, double a, int nmax, double eps) {
    if (damp == DAMP_NONE || !(a > 0.0)) return 0.0;
    nmax = std::min(nmax, 6);
    const int j0 = damp == DAMP_AMOEBA ? 1 : 0;
    double last_bad = 0.0;
    double g[7], g0[7];
    for (int k = 0; k <= 4000; ++k) {
        const double r = 1e-3 * std::pow(1e8, k / 4000.0);
        radial_g(damp, r, a, 6, g);
        radial_g(DAMP_NONE, r, a, 6, g0);
        double dev = 0.0;
        for (int j = j0; j <= nmax; ++j) dev = std::max(dev, std::fabs(g[j] - g0[j]) / std::fabs(g0[j]));
        if (dev > eps) last_bad = r;
    }
    return last_bad * std::pow(1e8, 1.0 / 4000.0);
}

// interact_fmm (fmm.F90:352-385): the source cell is displaced by g_disp
// (the periodic image's displacement, 0 otherwise).  With rdamp > 0 a pair
// that passes the reference test is still refused when its closest possible
// particle distance is inside the damping range.
double g_rdamp = 0.0;
double g_disp[3] = {0.0, 0.0, 0.0};
void interact(Tree& t, int i, int j, double theta) {
    const Node& a = t.nd[i];
    const Node& b = t.nd[j];
    double dx = a.c[0] - (b.c[0] + g_disp[0]);
    double dy = a.c[1] - (b.c[1] + g_disp[1]);
    double dz = a.c[2] - (b.c[2] + g_disp[2]);
    double r = norm2_3(dx, dy, dz);
    bool accept = r * theta > a.rmax + b.rmax;
    if (accept && g_rdamp > 0.0) accept = (r - 1.7320508075688772 * (a.r + b.r)) >= g_rdamp;
    if (accept) {
        t.far[a.idx].push_back(b.idx);
    } else if (a.terminal && b.terminal) {
        t.nearl[a.idx].push_back(b.idx);
    } else if (b.terminal || ((a.rmax > b.rmax) && !a.terminal)) {
        for (int o = 0; o < 8; ++o)
            if (a.child[o] >= 0) interact(t, a.child[o], j, theta);
    } else {
        for (int o = 0; o < 8; ++o)
            if (b.child[o] >= 0) interact(t, i, b.child[o], theta);
    }
}

void build_lists(Tree& t, double theta, double rdamp = 0.0, const double* disp = nullptr) {
    g_rdamp = rdamp;
    for (int c = 0; c < 3; ++c) g_disp[c] = disp ? disp[c] : 0.0;
    size_t M = t.nd.size();
    t.far.assign(M, {});
    t.nearl.assign(M, {});
    interact(t, 0, 0, theta);
}

struct Problem {
    int64_t n;
    const double* X;
    int dim;
    const double* mp;
    int exw;
    const int32_t* ex;
    int pf;
    int damp;
    const double* dampf;
};

int nthreads_of(const OracleOpts* o) {
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
    if (o && o->nthreads > 0) nt = o->nthreads;
#else
    (void)o;
#endif
    return nt;
}

bool is_excluded(const Problem& P, int64_t i, int64_t j) {
    for (int w = 0; w < P.exw; ++w)
        if ((int64_t)P.ex[(size_t)w * P.n + i] == j + 1) return true;
    return false;
}

// particle_fields_direct (fmm.F90:749-824)
void direct_sum(const Problem& P, const Ctx& ctx, double* field, int nthreads) {
    int64_t n = P.n;
    int nf = nT(P.pf);
#pragma omp parallel num_threads(nthreads)
    {
        std::vector<double> x(n), y(n), z(n), a(n), M, Tb, F(nf);
        std::vector<int64_t> keep;
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < n; ++i) {
            int64_t ns = 0;
            keep.clear();
            if (ctx.excl_mode == 0) {
                for (int64_t j = 0; j < n; ++j) {
                    x[j] = P.X[i] - P.X[j];
                    y[j] = P.X[n + i] - P.X[n + j];
                    z[j] = P.X[2 * n + i] - P.X[2 * n + j];
                }
                for (int w = 0; w < P.exw; ++w) {
                    int e = P.ex[(size_t)w * n + i];
                    if (e == 0) continue;
                    x[e - 1] = 1e10;
                    y[e - 1] = 1e10;
                    z[e - 1] = 1e10;
                }
                ns = n;
                for (int64_t j = 0; j < n; ++j) keep.push_back(j);
            } else {
                for (int64_t j = 0; j < n; ++j) {
                    if (j == i || is_excluded(P, i, j)) continue;
                    x[ns] = P.X[i] - P.X[j];
                    y[ns] = P.X[n + i] - P.X[n + j];
                    z[ns] = P.X[2 * n + i] - P.X[2 * n + j];
                    keep.push_back(j);
                    ++ns;
                }
            }
            M.resize((size_t)ns * P.dim);
            for (int c = 0; c < P.dim; ++c)
                for (int64_t s = 0; s < ns; ++s) M[(size_t)c * ns + s] = P.mp[(size_t)c * n + keep[s]];
            if (P.damp != DAMP_NONE)
                for (int64_t s = 0; s < ns; ++s) a[s] = P.dampf[i] * P.dampf[keep[s]];
            multipole_field((int)ns, M.data(), P.dim, x.data(), y.data(), z.data(), P.pf, P.damp, a.data(), ctx, F.data(), Tb);
            for (int q = 0; q < nf; ++q) field[(size_t)q * n + i] = field[(size_t)q * n + i] + F[q];
        }
    }
}

// multipole_expansion (fmm.F90:474-546): P2M of every leaf
// (shift_multipole_vec, :437-472) and each leaf's moments translated straight
// into every ancestor (multipole_accumulate, :387-435); raw Cartesian moments,
// column-major (M, nT(p)).
std::vector<double> multipole_expansion(const Problem& P, const Tree& t, int p, const std::vector<int>& term) {
    const int64_t n = P.n;
    const int M = (int)t.nd.size(), ms = nT(p), pm = dim_to_order(P.dim);
    std::vector<double> cm((size_t)M * ms, 0.0);  // (M, ms) column-major
    for (int d : term) {
        const Node& nd = t.nd[t.dfs[d]];
        int nl = nd.nleaf;
        std::vector<double> dx(nl), dy(nl), dz(nl);
        for (int q = 0; q < nl; ++q) {
            dx[q] = P.X[nd.leaf[q]] - nd.c[0];
            dy[q] = P.X[n + nd.leaf[q]] - nd.c[1];
            dz[q] = P.X[2 * n + nd.leaf[q]] - nd.c[2];
        }
        // shift_multipole_vec (fmm.F90:437-472)
        for (int so = 0; so <= pm; ++so)
            for (int to = so; to <= p; ++to)
                for (int sx = so; sx >= 0; --sx)
                    for (int sy = so; sy >= 0; --sy)
                        for (int sz = so; sz >= 0; --sz) {
                            if (sx + sy + sz != so) continue;
                            int si = pidx(sx, sy, sz);
                            for (int tx = to; tx >= sx; --tx)
                                for (int ty = to; ty >= sy; --ty)
                                    for (int tz = to; tz >= sz; --tz) {
                                        if (tx + ty + tz != to) continue;
                                        int ti = pidx(tx, ty, tz);
                                        double symfac = (binom(tx, sx) * binom(ty, sy)) * binom(tz, sz);
                                        double sum = 0.0;
                                        for (int q = 0; q < nl; ++q) {
                                            double mono = (ipow(dx[q], tx - sx) * ipow(dy[q], ty - sy)) * ipow(dz[q], tz - sz);
                                            sum = sum + mono * P.mp[(size_t)si * n + nd.leaf[q]];
                                        }
                                        cm[(size_t)ti * M + d] = cm[(size_t)ti * M + d] + symfac * sum;
                                    }
                        }
    }
    // multipole_accumulate: each leaf straight into every ancestor, root first
    auto m2m_kernel = [&](int src, int dst) {
        const Node& s = t.nd[t.dfs[src]];
        const Node& g = t.nd[t.dfs[dst]];
        double del[3] = {s.c[0] - g.c[0], s.c[1] - g.c[1], s.c[2] - g.c[2]};
        for (int so = 0; so <= p; ++so)
            for (int to = so; to <= p; ++to)
                for (int sx = so; sx >= 0; --sx)
                    for (int sy = so; sy >= 0; --sy)
                        for (int sz = so; sz >= 0; --sz) {
                            if (sx + sy + sz != so) continue;
                            int si = pidx(sx, sy, sz);
                            for (int tx = to; tx >= sx; --tx)
                                for (int ty = to; ty >= sy; --ty)
                                    for (int tz = to; tz >= sz; --tz) {
                                        if (tx + ty + tz != to) continue;
                                        int ti = pidx(tx, ty, tz);
                                        double symfac = (binom(tx, sx) * binom(ty, sy)) * binom(tz, sz);
                                        double mono = (ipow(del[0], tx - sx) * ipow(del[1], ty - sy)) * ipow(del[2], tz - sz);
                                        cm[(size_t)ti * M + dst] = cm[(size_t)ti * M + dst] + (symfac * mono) * cm[(size_t)si * M + src];
                                    }
                        }
    };
    for (int d : term) {
        std::vector<int> anc;
        int ci = t.nd[t.dfs[d]].parent;
        while (ci >= 0) {
            anc.push_back(t.nd[ci].idx);
            ci = t.nd[ci].parent;
        }
        for (int q = (int)anc.size() - 1; q >= 0; --q) m2m_kernel(d, anc[q]);
    }
    return cm;
}

// local_to_local (fmm.F90:981-1044), depth by depth, then local_to_particle
// (fmm.F90:1046-1132) into field (n x nT(P.pf), accumulated).
void local_to_local_and_particle(const Problem& P, const Tree& t, int p, const std::vector<int>& term,
                                 std::vector<double>& loc, double* field, int nthreads) {
    const int64_t n = P.n;
    const int M = (int)t.nd.size();
    // --- local_to_local (fmm.F90:981-1044), depth by depth
    for (int depth = 2; depth <= t.max_depth; ++depth) {
        for (int d = 0; d < M; ++d) {
            const Node& nd = t.nd[t.dfs[d]];
            if (nd.depth != depth) continue;
            int par = t.nd[nd.parent].idx;
            double dx = nd.c[0] - t.nd[nd.parent].c[0];
            double dy = nd.c[1] - t.nd[nd.parent].c[1];
            double dz = nd.c[2] - t.nd[nd.parent].c[2];
            for (int to = 0; to <= p; ++to)
                for (int tx = to; tx >= 0; --tx)
                    for (int ty = to; ty >= 0; --ty)
                        for (int tz = to; tz >= 0; --tz) {
                            if (tx + ty + tz != to) continue;
                            int ti = pidx(tx, ty, tz);
                            for (int so = to; so <= p; ++so)
                                for (int sx = so; sx >= tx; --sx)
                                    for (int sy = so; sy >= ty; --sy)
                                        for (int sz = so; sz >= tz; --sz) {
                                            if (sx + sy + sz != so) continue;
                                            int si = pidx(sx, sy, sz);
                                            double pre = 1.0 / ((factorial(sx - tx) * factorial(sy - ty)) * factorial(sz - tz));
                                            double mono = (ipow(dx, sx - tx) * ipow(dy, sy - ty)) * ipow(dz, sz - tz);
                                            loc[(size_t)ti * M + d] = loc[(size_t)ti * M + d] + (pre * loc[(size_t)si * M + par]) * mono;
                                        }
                        }
        }
    }
    // --- local_to_particle (fmm.F90:1046-1132)
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 8)
    for (size_t ti2 = 0; ti2 < term.size(); ++ti2) {
        int d = term[ti2];
        const Node& nd = t.nd[t.dfs[d]];
        for (int q = 0; q < nd.nleaf; ++q) {
            int64_t i = nd.leaf[q];
            double dx = P.X[i] - nd.c[0], dy = P.X[n + i] - nd.c[1], dz = P.X[2 * n + i] - nd.c[2];
            for (int to = 0; to <= P.pf; ++to)
                for (int tx = to; tx >= 0; --tx)
                    for (int ty = to; ty >= 0; --ty)
                        for (int tz = to; tz >= 0; --tz) {
                            if (tx + ty + tz != to) continue;
                            int ti = pidx(tx, ty, tz);
                            for (int so = to; so <= p; ++so)
                                for (int sx = so; sx >= tx; --sx)
                                    for (int sy = so; sy >= ty; --sy)
                                        for (int sz = so; sz >= tz; --sz) {
                                            if (sx + sy + sz != so) continue;
                                            int si = pidx(sx, sy, sz);
                                            double pre = 1.0 / ((factorial(sx - tx) * factorial(sy - ty)) * factorial(sz - tz));
                                            double v = (((pre * loc[(size_t)si * M + d]) * ipow(dx, sx - tx)) * ipow(dy, sy - ty)) * ipow(dz, sz - tz);
                                            field[(size_t)ti * n + i] = field[(size_t)ti * n + i] + v;
                                        }
                        }
        }
    }
}

// NORM2 of a vector with the scaled sum of squares.
double norm2_n(const double* v, int len) {
    double scale = 0.0, ssq = 1.0;
    for (int i = 0; i < len; ++i) {
        if (v[i] != 0.0) {
            double ax = std::fabs(v[i]);
            if (scale < ax) {
                double t = scale / ax;
                ssq = 1.0 + (ssq * t) * t;
                scale = ax;
            } else {
                double t = ax / scale;
                ssq = ssq + t * t;
            }
        }
    }
    return scale * std::sqrt(ssq);
}

// displacement = matmul(box, a) for an integer-valued vector a (fmm.F90:355)
void box_times(const double* box, const double* a, double* out) {
    for (int i = 0; i < 3; ++i) out[i] = (box[i] * a[0] + box[3 + i] * a[1]) + box[6 + i] * a[2];
}

// lattice levels used by the last periodic call (diagnostics)
int g_lattice_levels = 0;

// periodic_sum (fmm.F90:884-952): the lattice beyond the 27 images, in 3x3x3
// supercells, into the root's local expansion; then dipole_correction
// (fmm.F90:954-979) on the field.  In exact mode the level's tensors are
// evaluated at R 2^-k (k ~ level log2 3; scaling by a power of two is exact)
// with the moments and the result rescaled to match, so orders up to 2p do
// not underflow at the far levels; ref mode is the reference's arithmetic.
void periodic_sum_and_surface(const Problem& P, const Tree& t, int p, Ctx& ctx, std::vector<double>& cm,
                              std::vector<double>& loc, const double* box, double* field) {
    const int64_t n = P.n;
    const int M = (int)t.nd.size(), ms = nT(p);
    const int root = 0;
    cm[(size_t)0 * M + root] = 0.0;  // the reference forces charge neutrality
    const int K = 26 * 27;
    std::vector<double> S(ms), scaled(ms), contrib(ms), Mb((size_t)K * ms), x(K), y(K), z(K), Tb;
    for (int c = 0; c < ms; ++c) S[c] = scaled[c] = cm[(size_t)c * M + root];
    ctx.ensure_cnij(2 * p);
    const bool ref = ctx.coef_mode == 0;
    g_lattice_levels = 0;
    for (int level = 1; level <= 50; ++level) {
        int k = 0;
        for (int ai = -1; ai <= 1; ++ai)
            for (int aj = -1; aj <= 1; ++aj)
                for (int ak = -1; ak <= 1; ++ak) {
                    if (ai == 0 && aj == 0 && ak == 0) continue;
                    const double p3 = ipow(3.0, level), p3m = ipow(3.0, level - 1);
                    const double aijk[3] = {ai * p3, aj * p3, ak * p3};
                    double da[3], del[3];
                    box_times(box, aijk, da);
                    for (int c = 0; c < 3; ++c) del[c] = da[c] / 3.0;
                    // multipole_accumulate_kernel(d_aijk / 3, S, scaled) (fmm.F90:387-416)
                    for (int so = 0; so <= p; ++so)
                        for (int to = so; to <= p; ++to)
                            for (int sx = so; sx >= 0; --sx)
                                for (int sy = so; sy >= 0; --sy)
                                    for (int sz = so; sz >= 0; --sz) {
                                        if (sx + sy + sz != so) continue;
                                        int si = pidx(sx, sy, sz);
                                        for (int tx = to; tx >= sx; --tx)
                                            for (int ty = to; ty >= sy; --ty)
                                                for (int tz = to; tz >= sz; --tz) {
                                                    if (tx + ty + tz != to) continue;
                                                    int ti = pidx(tx, ty, tz);
                                                    double symfac = (binom(tx, sx) * binom(ty, sy)) * binom(tz, sz);
                                                    double mono = (ipow(del[0], tx - sx) * ipow(del[1], ty - sy)) *
                                                                  ipow(del[2], tz - sz);
                                                    scaled[ti] = scaled[ti] + (symfac * mono) * S[si];
                                                }
                                    }
                    for (int bi = -1; bi <= 1; ++bi)
                        for (int bj = -1; bj <= 1; ++bj)
                            for (int bk = -1; bk <= 1; ++bk) {
                                const double bijk[3] = {bi * p3m, bj * p3m, bk * p3m};
                                double db[3];
                                box_times(box, bijk, db);
                                x[k] = da[0] + db[0];
                                y[k] = da[1] + db[1];
                                z[k] = da[2] + db[2];
                                ++k;
                            }
                }
        const int ksc = ref ? 0 : (int)std::floor(level * 1.5849625007211563);
        for (int c = 0; c < ms; ++c)
            for (int q = 0; q < K; ++q) Mb[(size_t)c * K + q] = std::ldexp(S[c], -ksc * order_of(c));
        for (int q = 0; q < K; ++q) {
            x[q] = std::ldexp(x[q], -ksc);
            y[q] = std::ldexp(y[q], -ksc);
            z[q] = std::ldexp(z[q], -ksc);
        }
        multipole_field(K, Mb.data(), ms, x.data(), y.data(), z.data(), p, DAMP_NONE, nullptr, ctx, contrib.data(), Tb);
        for (int c = 0; c < ms; ++c) contrib[c] = std::ldexp(contrib[c], -ksc * (order_of(c) + 1));
        for (int c = 0; c < ms; ++c) loc[(size_t)c * M + root] = loc[(size_t)c * M + root] + contrib[c];
        S = scaled;
        g_lattice_levels = level;
        if (norm2_n(contrib.data() + 1, ms - 1) < 1.0e-8) break;
    }
    // --- dipole_correction (fmm.F90:954-979)
    auto h = [&](int i, int j) { return box[(j - 1) * 3 + (i - 1)]; };
    const double vol =
        ref ? h(1, 1) * (h(2, 2) * h(3, 3) - h(2, 3) * h(3, 2)) - h(1, 2) * (h(2, 1) * h(3, 3) - h(2, 3) * h(3, 1)) +
                  h(1, 3) * (h(1, 2) * h(3, 2) - h(2, 2) * h(3, 1))
            : h(1, 1) * (h(2, 2) * h(3, 3) - h(2, 3) * h(3, 2)) - h(1, 2) * (h(2, 1) * h(3, 3) - h(2, 3) * h(3, 1)) +
                  h(1, 3) * (h(2, 1) * h(3, 2) - h(2, 2) * h(3, 1));
    const double pi = ref ? 3.14159265359 : M_PI;
    const double dip[3] = {cm[(size_t)1 * M + root], cm[(size_t)2 * M + root], cm[(size_t)3 * M + root]};
    const double qtr = (cm[(size_t)4 * M + root] + cm[(size_t)7 * M + root]) + cm[(size_t)9 * M + root];
    for (int64_t i = 0; i < n; ++i) {
        const double dot = (dip[0] * P.X[i] + dip[1] * P.X[n + i]) + dip[2] * P.X[2 * n + i];
        field[i] = (field[i] + 4.0 * pi * dot / (3.0 * vol)) + 2.0 * pi * qtr / (3.0 * vol);
    }
    if (P.pf >= 1)
        for (int64_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c)
                field[(size_t)(1 + c) * n + i] = field[(size_t)(1 + c) * n + i] + 4.0 * pi * dip[c] / (3.0 * vol);
}

int run_fmm(const Problem& P, double theta, int ncrit, int p, const Ctx& ctx0, double* field, int nthreads,
            const double* box = nullptr) {
    Ctx ctx = ctx0;
    int64_t n = P.n;
    int nf = nT(P.pf);
    int pm = dim_to_order(P.dim);
    Tree t;
    int st = build_tree(P.X, n, ncrit, ctx.centroid_mode, t);
    if (st) return st;
    double rdamp = 0.0;
    if (ctx.mac_mode == 1 && P.damp != DAMP_NONE) {
        double dmin = 1e300;
        for (int64_t q = 0; q < n; ++q) dmin = std::min(dmin, P.dampf[q]);
        rdamp = damping_range(P.damp, dmin * dmin, pm + P.pf, 0.1 * ctx.target);
    }
    build_lists(t, theta, rdamp);
    const int nimg = box ? 27 : 1;
    int M = (int)t.nd.size();
    int ms = nT(p);
    // leaf id of every particle
    std::vector<int> leaf_of(n, -1);
    std::vector<int> term;
    for (int d = 0; d < M; ++d) {
        const Node& nd = t.nd[t.dfs[d]];
        if (!nd.terminal) continue;
        term.push_back(d);
        for (int q = 0; q < nd.nleaf; ++q) leaf_of[nd.leaf[q]] = d;
    }
    std::vector<double> cm = multipole_expansion(P, t, p, term);
    std::vector<double> loc((size_t)M * ms, 0.0);
    // periodic boxes: the 27 images (a_x outer, a_z inner; fmm.F90:156-175),
    // each with its own lists; exclusions only in the central image
    for (int img = 0; img < nimg; ++img) {
        double disp[3] = {0.0, 0.0, 0.0};
        bool central = true;
        if (box) {
            const double av[3] = {(double)(img / 9 - 1), (double)((img / 3) % 3 - 1), (double)(img % 3 - 1)};
            box_times(box, av, disp);
            central = img == 13;
            build_lists(t, theta, rdamp, disp);
        }
        // --- particle_fields (fmm.F90:623-747)
        {
            ctx.ensure_cnij(pm + P.pf);
    #pragma omp parallel num_threads(nthreads)
            {
                std::vector<double> x, y, z, a, Mb, Tb, F(nf);
    #pragma omp for schedule(dynamic, 4)
                for (size_t ti = 0; ti < term.size(); ++ti) {
                    int d = term[ti];
                    const Node& ndi = t.nd[t.dfs[d]];
                    for (int q = 0; q < ndi.nleaf; ++q) {
                        int64_t i = ndi.leaf[q];
                        for (int dj : t.nearl[d]) {
                            const Node& ndj = t.nd[t.dfs[dj]];
                            int nl = ndj.nleaf;
                            x.resize(nl);
                            y.resize(nl);
                            z.resize(nl);
                            a.resize(nl);
                            std::vector<int> src;
                            src.reserve(nl);
                            for (int w = 0; w < nl; ++w) {
                                int64_t j = ndj.leaf[w];
                                if (central && ctx.excl_mode == 1 && (j == i || is_excluded(P, i, j))) continue;
                                size_t s = src.size();
                                x[s] = P.X[i] - (P.X[j] + disp[0]);
                                y[s] = P.X[n + i] - (P.X[n + j] + disp[1]);
                                z[s] = P.X[2 * n + i] - (P.X[2 * n + j] + disp[2]);
                                if (central && ctx.excl_mode == 0 && is_excluded(P, i, j)) x[s] = y[s] = z[s] = 1e10;
                                if (P.damp != DAMP_NONE) a[s] = P.dampf[i] * P.dampf[j];
                                src.push_back((int)j);
                            }
                            int ns = (int)src.size();
                            Mb.resize((size_t)ns * P.dim);
                            for (int c = 0; c < P.dim; ++c)
                                for (int s = 0; s < ns; ++s) Mb[(size_t)c * ns + s] = P.mp[(size_t)c * n + src[s]];
                            multipole_field(ns, Mb.data(), P.dim, x.data(), y.data(), z.data(), P.pf, P.damp, a.data(), ctx, F.data(), Tb);
                            for (int c = 0; c < nf; ++c) field[(size_t)c * n + i] = field[(size_t)c * n + i] + F[c];
                        }
                        if (central && ctx.excl_mode == 1) {
                            // far-field exclusion correction: excluded partners whose
                            // leaf is not a near leaf were counted through M2L; take
                            // their undamped pair field out again.
                            for (int w = 0; w < P.exw; ++w) {
                                int e = P.ex[(size_t)w * n + i];
                                if (e == 0 || e - 1 == i) continue;
                                bool dup = false;
                                for (int w2 = 0; w2 < w; ++w2)
                                    if (P.ex[(size_t)w2 * n + i] == e) dup = true;
                                if (dup) continue;
                                int lj = leaf_of[e - 1];
                                const auto& nl = t.nearl[d];
                                if (std::find(nl.begin(), nl.end(), lj) != nl.end()) continue;
                                int64_t j = e - 1;
                                double xx = P.X[i] - P.X[j], yy = P.X[n + i] - P.X[n + j], zz = P.X[2 * n + i] - P.X[2 * n + j];
                                Mb.resize(P.dim);
                                for (int c = 0; c < P.dim; ++c) Mb[c] = P.mp[(size_t)c * n + j];
                                multipole_field(1, Mb.data(), P.dim, &xx, &yy, &zz, P.pf, DAMP_NONE, nullptr, ctx, F.data(), Tb);
                                for (int c = 0; c < nf; ++c) field[(size_t)c * n + i] = field[(size_t)c * n + i] - F[c];
                            }
                        }
                    }
                }
            }
        }
        // --- multipole_to_local (fmm.F90:826-882)
        {
            ctx.ensure_cnij(2 * p);
    #pragma omp parallel num_threads(nthreads)
            {
                std::vector<double> x, y, z, Mb, Tb, F(ms);
    #pragma omp for schedule(dynamic, 1)
                for (int d = 0; d < M; ++d) {
                    const auto& fl = t.far[d];
                    int nl = (int)fl.size();
                    const Node& ndi = t.nd[t.dfs[d]];
                    x.resize(nl);
                    y.resize(nl);
                    z.resize(nl);
                    Mb.resize((size_t)nl * ms);
                    for (int q = 0; q < nl; ++q) {
                        const Node& ndj = t.nd[t.dfs[fl[q]]];
                        x[q] = ndi.c[0] - (ndj.c[0] + disp[0]);
                        y[q] = ndi.c[1] - (ndj.c[1] + disp[1]);
                        z[q] = ndi.c[2] - (ndj.c[2] + disp[2]);
                        for (int c = 0; c < ms; ++c) Mb[(size_t)c * nl + q] = cm[(size_t)c * M + fl[q]];
                    }
                    multipole_field(nl, Mb.data(), ms, x.data(), y.data(), z.data(), p, DAMP_NONE, nullptr, ctx, F.data(), Tb);
                    for (int c = 0; c < ms; ++c) loc[(size_t)c * M + d] = loc[(size_t)c * M + d] + F[c];
                }
            }
        }
    }
    if (box) periodic_sum_and_surface(P, t, p, ctx, cm, loc, box, field);
    local_to_local_and_particle(P, t, p, term, loc, field, nthreads);
    return OK;
}

int parse_common(int64_t n, int dim, int exw, const int32_t* ex, int pf, int damp, const double* dampf) {
    if (n < 1 || pf < 0 || exw < 0) return E_INVAL;
    if (dim_to_order(dim) < 0) return E_INVAL;
    if (damp < 0 || damp > 3) return E_INVAL;
    if (damp != DAMP_NONE && !dampf) return E_INVAL;
    for (int64_t q = 0; q < n * (int64_t)exw; ++q)
        if (ex[q] < 0 || ex[q] > n) return E_INVAL;
    return OK;
}

Ctx make_ctx(const OracleOpts* o) {
    Ctx c;
    if (o) {
        c.coef_mode = o->coef_mode;
        c.excl_mode = o->excl_mode;
        c.centroid_mode = o->centroid_mode;
        c.mac_mode = o->mac_mode;
        c.target = o->target_rel_err > 0 ? o->target_rel_err : 1e-6;
    }
    return c;
}

struct TreeHandle {
    Tree t;
    std::vector<int> leaf_of;
};

}  // namespace

extern "C" {

// T tensors of every order <= nmax for ns displacements (column-major (ns, nT(nmax))).
int oracle_tensors(int nmax, int64_t ns, const double* x, const double* y, const double* z, int damp, const double* a,
                   int coef_mode, double* T) {
    if (nmax < 0 || ns < 0) return E_INVAL;
    Ctx c;
    c.coef_mode = coef_mode;
    if (damp == DAMP_NONE) c.ensure_cnij(std::max(nmax, 1));
    tensors(nmax, (int)ns, x, y, z, damp, a, c, T);
    return OK;
}

int oracle_radial_g(int damp, double r, double a, int n, double* g) {
    radial_g(damp, r, a, n, g);
    return OK;
}

int oracle_field_direct(int64_t n, const double* coords, int dim, const double* mp, int exw, const int32_t* ex,
                        int field_order, double* field, int damp, const double* dampf, const OracleOpts* opts) {
    int st = parse_common(n, dim, exw, ex, field_order, damp, dampf);
    if (st) return st;
    Ctx ctx = make_ctx(opts);
    ctx.ensure_cnij(std::max(1, dim_to_order(dim) + field_order));
    Problem P{n, coords, dim, mp, exw, ex, field_order, damp, dampf};
    std::memset(field, 0, sizeof(double) * (size_t)n * nT(field_order));
    direct_sum(P, ctx, field, nthreads_of(opts));
    return OK;
}

int oracle_field_fmm_box(int64_t n, const double* coords, int dim, const double* mp, int exw, const int32_t* ex,
                         double theta, int ncrit, int expansion_order, int field_order, double* field, int damp,
                         const double* dampf, int is_periodic, const double* box, const OracleOpts* opts) {
    int st = parse_common(n, dim, exw, ex, field_order, damp, dampf);
    if (st) return st;
    if (ncrit < 1 || expansion_order < 0 || !(theta > 0.0)) return E_INVAL;
    if (is_periodic && (!box || n <= ncrit)) return E_INVAL;  // the reference stops (fmm.F90:1382)
    if (n <= ncrit) return oracle_field_direct(n, coords, dim, mp, exw, ex, field_order, field, damp, dampf, opts);
    Ctx ctx = make_ctx(opts);
    ctx.ensure_cnij(std::max(1, dim_to_order(dim) + field_order));
    Problem P{n, coords, dim, mp, exw, ex, field_order, damp, dampf};
    std::memset(field, 0, sizeof(double) * (size_t)n * nT(field_order));
    return run_fmm(P, theta, ncrit, expansion_order, ctx, field, nthreads_of(opts), is_periodic ? box : nullptr);
}

int oracle_field_fmm(int64_t n, const double* coords, int dim, const double* mp, int exw, const int32_t* ex,
                     double theta, int ncrit, int expansion_order, int field_order, double* field, int damp,
                     const double* dampf, int is_periodic, const OracleOpts* opts) {
    if (is_periodic) return E_INVAL;  // needs the box: oracle_field_fmm_box
    return oracle_field_fmm_box(n, coords, dim, mp, exw, ex, theta, ncrit, expansion_order, field_order, field, damp,
                                dampf, 0, nullptr, opts);
}

// Tree + lists of the reference construction, for integer comparisons.
void* oracle_tree_build(int64_t n, const double* coords, int ncrit, double theta, int centroid_mode, int* status) {
    auto* h = new TreeHandle();
    int st = build_tree(coords, n, ncrit, centroid_mode, h->t);
    if (st) {
        *status = st;
        delete h;
        return nullptr;
    }
    build_lists(h->t, theta);
    *status = OK;
    return h;
}

void oracle_tree_sizes(void* hp, int64_t* out /* [num_nodes, nfar, nnear, max_depth] */) {
    auto* h = (TreeHandle*)hp;
    int64_t nf = 0, nn = 0;
    for (auto& v : h->t.far) nf += (int64_t)v.size();
    for (auto& v : h->t.nearl) nn += (int64_t)v.size();
    out[0] = (int64_t)h->t.nd.size();
    out[1] = nf;
    out[2] = nn;
    out[3] = h->t.max_depth;
}

// Per DFS node: centre (3), r, rmax, depth, parent dfs id (-1 for the root),
// is_leaf, particle count; per particle: leaf dfs id; far/near lists as
// (target, source) dfs id pairs, sorted.
void oracle_tree_get(void* hp, double* center /*3M*/, double* r, double* rmax, int32_t* depth, int32_t* parent,
                     int32_t* is_leaf, int32_t* count, int32_t* leaf_of /*n*/, int32_t* far_pairs /*2*nfar*/,
                     int32_t* near_pairs /*2*nnear*/) {
    auto* h = (TreeHandle*)hp;
    Tree& t = h->t;
    int M = (int)t.nd.size();
    for (int d = 0; d < M; ++d) {
        const Node& nd = t.nd[t.dfs[d]];
        center[3 * d + 0] = nd.c[0];
        center[3 * d + 1] = nd.c[1];
        center[3 * d + 2] = nd.c[2];
        r[d] = nd.r;
        rmax[d] = nd.rmax;
        depth[d] = nd.depth;
        parent[d] = nd.parent >= 0 ? t.nd[nd.parent].idx : -1;
        is_leaf[d] = nd.terminal ? 1 : 0;
        count[d] = nd.nleaf;
        if (nd.terminal)
            for (int q = 0; q < nd.nleaf; ++q) leaf_of[nd.leaf[q]] = d;
    }
    std::vector<std::pair<int, int>> fp, np;
    for (int d = 0; d < M; ++d) {
        for (int s : t.far[d]) fp.push_back({d, s});
        for (int s : t.nearl[d]) np.push_back({d, s});
    }
    std::sort(fp.begin(), fp.end());
    std::sort(np.begin(), np.end());
    for (size_t q = 0; q < fp.size(); ++q) {
        far_pairs[2 * q] = fp[q].first;
        far_pairs[2 * q + 1] = fp[q].second;
    }
    for (size_t q = 0; q < np.size(); ++q) {
        near_pairs[2 * q] = np[q].first;
        near_pairs[2 * q + 1] = np[q].second;
    }
}

void oracle_tree_free(void* hp) { delete (TreeHandle*)hp; }

// ---------------------------------------------------------------- QM/MM helpers
// classify_box (fmm.F90:1134-1171): a node with a target within rmax / theta
// of its centre is refined (a leaf: its particles are used), otherwise its
// box multipole is used.  type[DFS id]: 0 unused, 1 box, 2 particles.
void classify(const Tree& t, int b, const double* tc, int64_t ntgt, double theta, std::vector<int>& type) {
    const Node& nd = t.nd[b];
    bool too_close = false;
    for (int64_t i = 0; i < ntgt; ++i) {
        double r = norm2_3(tc[i] - nd.c[0], tc[ntgt + i] - nd.c[1], tc[2 * ntgt + i] - nd.c[2]);
        if (r * theta <= nd.rmax) too_close = true;
    }
    if (too_close && !nd.terminal) {
        for (int o = 0; o < 8; ++o)
            if (nd.child[o] >= 0) classify(t, nd.child[o], tc, ntgt, theta, type);
    } else if (too_close && nd.terminal) {
        type[nd.idx] = 2;
    } else {
        type[nd.idx] = 1;
    }
}

// The outputs of get_boxes / get_multipoles that depend on the tree only
// (fmm.F90:1173-1233, 1258-1308): near-field particles (1-based, node
// order, leaf order) and the boxes (centres, 1-based DFS ids).
void boxes_of(const Tree& t, const std::vector<int>& type, int64_t* sizes, int32_t* idx_near, double* box_c,
              int32_t* box_idx) {
    const int M = (int)t.nd.size();
    int64_t nn = 0, nb = 0;
    for (int d = 0; d < M; ++d) {
        const Node& nd = t.nd[t.dfs[d]];
        if (type[d] == 2) nn += nd.nleaf;
        if (type[d] == 1) ++nb;
    }
    sizes[0] = nn;
    sizes[1] = nb;
    int64_t k = 0, b = 0;
    for (int d = 0; d < M; ++d) {
        const Node& nd = t.nd[t.dfs[d]];
        if (type[d] == 2 && idx_near)
            for (int q = 0; q < nd.nleaf; ++q) idx_near[k++] = (int32_t)(nd.leaf[q] + 1);
        if (type[d] == 1) {
            if (box_c)
                for (int c = 0; c < 3; ++c) box_c[(size_t)c * nb + b] = nd.c[c];
            if (box_idx) box_idx[b] = d + 1;
            ++b;
        }
    }
}

// The Cnij coefficient table for tensors up to order maxo, in the layout of
// the reference's Cnij(1:2*maxo+3, 0:maxo+1, 0:maxo+1) (column-major;
// tensors_recursive.F90:64-93): wrap32 = 1 gives the int32 table of the
// default build, 0 the exact integers.
// get_boxes (fmm.F90:1258-1308).  sizes[0] = near-field particles, sizes[1]
// = boxes; outputs may be NULL (sizes only).
int oracle_get_boxes(int64_t n, const double* coords, int64_t ntgt, const double* tgt, double theta, int ncrit,
                     int64_t* sizes, int32_t* idx_near, double* box_c, int32_t* box_idx) {
    Tree t;
    int st = build_tree(coords, n, ncrit, 0, t);
    if (st) return st;
    std::vector<int> type(t.nd.size(), 0);
    classify(t, 0, tgt, ntgt, theta, type);
    boxes_of(t, type, sizes, idx_near, box_c, box_idx);
    return OK;
}

// get_multipoles (fmm.F90:1173-1256): as get_boxes, plus the raw Cartesian
// multipoles of the boxes for each of ndens multipole sets (box_mp: nbox x
// nT(p) x ndens, column-major; mp: n x dim x ndens).
int oracle_get_multipoles(int64_t n, const double* coords, int dim, int ndens, const double* mp, int64_t ntgt,
                          const double* tgt, double theta, int ncrit, int p, int64_t* sizes, int32_t* idx_near,
                          double* box_c, double* box_mp) {
    if (dim_to_order(dim) < 0 || ndens < 1) return E_INVAL;
    Tree t;
    int st = build_tree(coords, n, ncrit, 0, t);
    if (st) return st;
    std::vector<int> type(t.nd.size(), 0);
    classify(t, 0, tgt, ntgt, theta, type);
    boxes_of(t, type, sizes, idx_near, box_c, nullptr);
    if (!box_mp) return OK;
    const int M = (int)t.nd.size(), ms = nT(p);
    const int64_t nb = sizes[1];
    std::vector<int> term;
    for (int d = 0; d < M; ++d)
        if (t.nd[t.dfs[d]].terminal) term.push_back(d);
    for (int k = 0; k < ndens; ++k) {
        Problem P{n, coords, dim, mp + (size_t)k * n * dim, 0, nullptr, 0, DAMP_NONE, nullptr};
        std::vector<double> cm = multipole_expansion(P, t, p, term);
        int64_t b = 0;
        for (int d = 0; d < M; ++d) {
            if (type[d] != 1) continue;
            for (int c = 0; c < ms; ++c) box_mp[((size_t)k * ms + c) * nb + b] = cm[(size_t)c * M + d];
            ++b;
        }
    }
    return OK;
}

// interpolate_electron_fields (fmm.F90:1310-1336): local expansions given at
// boxes (1-based DFS ids, local: nbox x nT(p) x ndens) carried down the tree
// (L2L) and evaluated at the particles (L2P); field (n x nT(f) x ndens) is
// zeroed first (the reference only adds into it).
int oracle_interpolate_electron_fields(int64_t n, const double* coords, int64_t nbox, int ndens, const double* local,
                                       const int32_t* box_idx, double theta, int ncrit, int p, int f, double* field) {
    (void)theta;
    Tree t;
    int st = build_tree(coords, n, ncrit, 0, t);
    if (st) return st;
    const int M = (int)t.nd.size(), ms = nT(p), nf = nT(f);
    for (int64_t b = 0; b < nbox; ++b)
        if (box_idx[b] < 1 || box_idx[b] > M) return E_INVAL;
    std::vector<int> term;
    for (int d = 0; d < M; ++d)
        if (t.nd[t.dfs[d]].terminal) term.push_back(d);
    std::memset(field, 0, sizeof(double) * (size_t)n * nf * ndens);
    for (int k = 0; k < ndens; ++k) {
        std::vector<double> loc((size_t)M * ms, 0.0);
        for (int64_t b = 0; b < nbox; ++b)
            for (int c = 0; c < ms; ++c)
                loc[(size_t)c * M + (box_idx[b] - 1)] = local[((size_t)k * ms + c) * nbox + b];
        Problem P{n, coords, 1, nullptr, 0, nullptr, f, DAMP_NONE, nullptr};
        local_to_local_and_particle(P, t, p, term, loc, field + (size_t)k * n * nf, 1);
    }
    return OK;
}

int oracle_last_lattice_levels(void) { return g_lattice_levels; }

void oracle_cnij(int maxo, int wrap32, double* out) {
    Cnij t = make_cnij(maxo, wrap32 != 0);
    for (int j = 0; j < t.d1; ++j)
        for (int i = 0; i < t.d1; ++i)
            for (int n = 1; n <= t.d0; ++n) out[(size_t)(n - 1) + (size_t)t.d0 * ((size_t)i + (size_t)t.d1 * j)] = t.get(n, i, j);
}

}  // extern "C"

"""CPU checks of the identities the translation kernels rely on
(fmm_gb300/csrc/translate.cu), on random data in FP64:

* M2M and L2L as three one-dimensional shifts (z, y, x) of a dense
  expansion equal the direct convolutions with d^u/u! (reference
  src/fmm.F90:387-435 and 981-1044 translate by the same sums);
* P2M as per-power products A_s[u] = sum_i M'_s(i) d_i^u/u! followed by
  M'_t = sum_{s<=t} A_s[t-s] equals the direct P2M sum (src/fmm.F90:437-472).
"""
import math

import numpy as np
import pytest


def comps(p):
    return [(x, y, k - x - y) for k in range(p + 1) for x in range(k, -1, -1) for y in range(k - x, -1, -1)]


def scaled_powers(d, p):
    return [[d[ax] ** a / math.factorial(a) for a in range(p + 1)] for ax in range(3)]


@pytest.mark.parametrize("p", [3, 8, 12])
def test_m2m_as_three_shifts(p):
    rng = np.random.default_rng(p)
    cs = comps(p)
    idx = {c: i for i, c in enumerate(cs)}
    e = scaled_powers(rng.normal(size=3), p)
    M = rng.normal(size=len(cs))
    direct = np.array([sum(e[0][ux] * e[1][uy] * e[2][uz] * M[idx[(tx - ux, ty - uy, tz - uz)]]
                           for ux in range(tx + 1) for uy in range(ty + 1) for uz in range(tz + 1))
                       for (tx, ty, tz) in cs])
    P1 = p + 1
    X = np.zeros((P1, P1, P1))
    Y = np.zeros_like(X)
    for i, c in enumerate(cs):
        X[c] = M[i]
    for (x, y, z) in cs:
        Y[x, y, z] = sum(e[2][u] * X[x, y, z - u] for u in range(z + 1))
    for (x, y, z) in cs:
        X[x, y, z] = sum(e[1][u] * Y[x, y - u, z] for u in range(y + 1))
    shifted = np.array([sum(e[0][u] * X[x - u, y, z] for u in range(x + 1)) for (x, y, z) in cs])
    assert np.abs(shifted - direct).max() <= 1e-13 * np.abs(direct).max()


@pytest.mark.parametrize("p", [3, 8, 12])
def test_l2l_as_three_shifts(p):
    rng = np.random.default_rng(100 + p)
    cs = comps(p)
    idx = {c: i for i, c in enumerate(cs)}
    e = scaled_powers(rng.normal(size=3), p)
    L = rng.normal(size=len(cs))
    direct = np.array([sum(L[idx[(tx + ux, ty + uy, tz + uz)]] * e[0][ux] * e[1][uy] * e[2][uz]
                           for (ux, uy, uz) in cs if ux + uy + uz <= p - tx - ty - tz)
                       for (tx, ty, tz) in cs])
    P1 = p + 1
    X = np.zeros((P1, P1, P1))
    Y = np.zeros_like(X)
    Z = np.zeros_like(X)
    for i, c in enumerate(cs):
        X[c] = L[i]
    for (x, y, z) in cs:
        Y[x, y, z] = sum(e[2][u] * X[x, y, z + u] for u in range(p - x - y - z + 1))
    for (x, y, z) in cs:
        Z[x, y, z] = sum(e[1][u] * Y[x, y + u, z] for u in range(p - x - y - z + 1))
    shifted = np.array([sum(e[0][u] * Z[x + u, y, z] for u in range(p - x - y - z + 1)) for (x, y, z) in cs])
    assert np.abs(shifted - direct).max() <= 1e-13 * np.abs(direct).max()


@pytest.mark.parametrize("p,m", [(6, 2), (12, 2), (10, 1)])
def test_p2m_as_per_power_products(p, m):
    rng = np.random.default_rng(200 + p)
    cs = comps(p)
    idx = {c: i for i, c in enumerate(cs)}
    nm = len(comps(m))
    npart = 7
    D = rng.normal(size=(npart, 3)) * 0.7
    W = rng.normal(size=(npart, nm))  # scaled moments M'_s(i)
    direct = np.zeros(len(cs))
    for i in range(npart):
        e = scaled_powers(D[i], p)
        for q, (tx, ty, tz) in enumerate(cs):
            for s, (sx, sy, sz) in enumerate(cs[:nm]):
                if sx <= tx and sy <= ty and sz <= tz:
                    direct[q] += W[i, s] * e[0][tx - sx] * e[1][ty - sy] * e[2][tz - sz]
    A = np.zeros((len(cs), nm))
    for i in range(npart):
        e = scaled_powers(D[i], p)
        for u, (ux, uy, uz) in enumerate(cs):
            for s in range(nm):
                if sum(cs[s]) <= p - ux - uy - uz:  # |u| <= p - |s|
                    A[u, s] += W[i, s] * e[0][ux] * e[1][uy] * e[2][uz]
    via_a = np.array([sum(A[idx[(tx - sx, ty - sy, tz - sz)], s] for s, (sx, sy, sz) in enumerate(cs[:nm])
                          if sx <= tx and sy <= ty and sz <= tz) for (tx, ty, tz) in cs])
    assert np.abs(via_a - direct).max() <= 1e-13 * np.abs(direct).max()

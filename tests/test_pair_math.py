"""CPU check of the quadrupole-source contraction of the near field
(fmm_gb300/csrc/pair.cuh contract_q1, and its packed form contract_q1_x2 in
fmm_gb300/csrc/pair_x2.cuh with the off-diagonal second moments supplied
halved) against the full Cartesian contraction sum_s Mc_s T_{s+f} of the
reference's multipole_field (src/fmm.F90:596-620), with the oracle's
interaction tensors and radial functions, for every damping kind."""
import numpy as np
import pytest

import oracle


def pidx(x, y, z):
    k, yz = x + y + z, y + z
    return k * (k + 1) * (k + 2) // 6 + yz * (yz + 1) // 2 + z


SOURCES = [(x, y, k - x - y) for k in range(3) for x in range(k, -1, -1) for y in range(k - x, -1, -1)]
FIELDS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)]


def full_contraction(Mc, T):
    return np.array([sum(Mc[pidx(*s)] * T[pidx(s[0] + f[0], s[1] + f[1], s[2] + f[2])] for s in SOURCES)
                     for f in FIELDS])


def q1_halved(Mc, R, g, damped_potential):
    """contract_q1_x2: w = grad q / 2 from halved xy, xz, yz moments,
    q = R . w, and the gradient term w (2 g_2)."""
    X, Y, Z = R
    h = Mc.copy()
    h[5] *= 0.5
    h[6] *= 0.5
    h[8] *= 0.5
    tr = Mc[4] + Mc[7] + Mc[9]
    wx = h[4] * X + h[5] * Y + h[6] * Z
    wy = h[5] * X + h[7] * Y + h[8] * Z
    wz = h[6] * X + h[8] * Y + h[9] * Z
    q = X * wx + Y * wy + Z * wz
    dtr = Mc[1] * X + Mc[2] * Y + Mc[3] * Z + tr
    sc = Mc[0] * g[1] + dtr * g[2] + q * g[3]
    a0 = dtr * g[1] + q * g[2] + (0.0 if damped_potential else Mc[0] * g[0])
    g2d = 2.0 * g[2]
    return np.array([a0, X * sc + Mc[1] * g[1] + wx * g2d, Y * sc + Mc[2] * g[1] + wy * g2d,
                     Z * sc + Mc[3] * g[1] + wz * g2d])


@pytest.mark.parametrize("damp", ["", "THOLE", "AMOEBA", "ERF"])
def test_q1_contraction_with_halved_moments(damp):
    rng = np.random.default_rng(7)
    for _ in range(25):
        R = rng.normal(size=3) * rng.uniform(0.5, 8.0)
        a = rng.uniform(0.15, 0.6)
        Mc = rng.normal(size=10)
        T = oracle.tensors(3, R[0:1], R[1:2], R[2:3], damp, np.array([a]), coef="exact")[0]
        g = oracle.radial_g(damp, float(np.linalg.norm(R)), a, 3)
        ref = full_contraction(Mc, T)
        got = q1_halved(Mc, R, g, damp == "AMOEBA")
        scale = np.max(np.abs(ref)) + 1e-300
        assert np.max(np.abs(got - ref)) <= 1e-12 * scale, (damp, R, a)


def test_amoeba_damping_correction_numerators():
    """The near field's damping correction (pair_x2.cuh radial_g_x2<N, true>)
    evaluates g_damped - g_undamped of AMOEBA as e^{-u} Q_j(u) / r^(2j+1) with
    the Q_j of the closed form (csrc/gen_tables.py), and -1/r for the
    potential; checked against the oracle's two kernels."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fmm_gb300", "csrc"))
    import gen_tables
    Q = gen_tables.amoeba_q()
    rng = np.random.default_rng(9)
    for _ in range(40):
        a = rng.uniform(0.15, 0.6)
        r = rng.uniform(2.0, 20.0)
        u = (a * r) ** 3
        gd = oracle.radial_g("AMOEBA", r, a, 4)
        gu = oracle.radial_g("", r, a, 4)
        assert abs((gd[0] - gu[0]) - (-1.0 / r)) <= 1e-14 / r
        for j in range(1, 5):
            corr = np.exp(-u) * sum(float(c) * u ** d for d, c in enumerate(Q[j])) / r ** (2 * j + 1)
            scale = abs(gu[j])
            assert abs((gd[j] - gu[j]) - corr) <= 1e-12 * scale, (a, r, j)

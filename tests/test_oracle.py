"""Pins of the CPU oracle (no GPU needed).

The reference ships no tests or golden vectors and cannot be compiled here
(it is Fortran), so the oracle is pinned by: symbolic tensors (sympy, in
tests/golden/tensors_sympy.npz), analytic identities of the interaction
tensors, the theta -> 0 limit of field_fmm, and convergence in the expansion
order.
"""
import os

import numpy as np
import pytest

import oracle
from helpers import per_target_rel, rel_err, small_system

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tensors_sympy.npz")


def _scale(x, y, z, nmax):
    r = np.sqrt(x * x + y * y + z * z)
    out = []
    for k in range(nmax + 1):
        s = np.prod(np.arange(1, 2 * k, 2)) / r ** (k + 1) if k else 1 / r
        out += [s] * ((k + 1) * (k + 2) // 2)
    return np.array(out)


@pytest.mark.parametrize("damp", ["NONE", "THOLE", "ERF", "AMOEBA"])
@pytest.mark.parametrize("coef", ["ref", "exact"])
def test_tensors_against_sympy(damp, coef):
    rows = np.load(GOLD)[damp]
    for row in rows:
        x, y, z, a = row[:4]
        T = oracle.tensors(6, [x], [y], [z], "" if damp == "NONE" else damp, [a], coef=coef)[0]
        err = np.abs(T - row[4:]) / _scale(x, y, z, 6)
        assert err.max() < 2e-13, (damp, row[:4], err.max())


def test_tensors_traceless():
    rng = np.random.default_rng(0)
    x, y, z = rng.normal(size=(3, 20)) * 4
    T = oracle.tensors(10, x, y, z, "", coef="exact")

    def idx(a, b, c):
        k = a + b + c
        return k * (k + 1) * (k + 2) // 6 + ((b + c) * (b + c + 1)) // 2 + c

    for k in range(2, 11):
        for a in range(k - 1):
            for b in range(k - 1 - a):
                c = k - 2 - a - b
                lap = T[:, idx(a + 2, b, c)] + T[:, idx(a, b + 2, c)] + T[:, idx(a, b, c + 2)]
                scale = np.abs(T[:, idx(a + 2, b, c)]) + np.abs(T[:, idx(a, b, c + 2)]) + 1e-300
                assert np.max(np.abs(lap) / np.maximum(scale, np.abs(T).max(axis=1) * 1e-3)) < 1e-9


def test_int32_wrap_changes_order11_only():
    rng = np.random.default_rng(1)
    x, y, z = rng.normal(size=(3, 10)) * 3
    for n in (6, 10):
        assert np.array_equal(oracle.tensors(n, x, y, z, "", coef="ref"), oracle.tensors(n, x, y, z, "", coef="exact"))
    Tr = oracle.tensors(12, x, y, z, "", coef="ref")
    Te = oracle.tensors(12, x, y, z, "", coef="exact")
    hi = slice(oracle.n_components(10), None)
    assert np.max(np.abs(Tr[:, hi] - Te[:, hi])) > 1e-6 * np.max(np.abs(Te[:, hi]))


def test_theta_to_zero_equals_direct():
    s = small_system(500, 18.0, seed=2)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    D = oracle.field_direct(*args, 1)
    F = oracle.field_fmm(*args, 1e-3, 16, 4, 1)
    assert rel_err(F, D) < 1e-13


def test_expansion_order_convergence_exact_mode():
    s = small_system(1500, 26.0, seed=3)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    D = oracle.field_direct(*args, 1, excl_mode="mask")
    errs = []
    for p in (3, 5, 8):
        F = oracle.field_fmm(*args, 0.5, 32, p, 1, coef_mode="exact", excl_mode="mask")
        errs.append(np.sqrt(np.mean(per_target_rel(F, D, slice(1, 4)) ** 2)))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 3e-4


def test_reference_far_field_keeps_excluded_pairs():
    """Reference mode counts excluded pairs that land in the far field; mask
    mode removes them, so it is closer to the direct sum."""
    s = small_system(1500, 26.0, seed=4)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    D = oracle.field_direct(*args, 1, excl_mode="mask")
    Fr = oracle.field_fmm(*args, 0.5, 32, 8, 1, coef_mode="exact")
    Fm = oracle.field_fmm(*args, 0.5, 32, 8, 1, coef_mode="exact", excl_mode="mask")
    assert rel_err(Fm, D, slice(1, 4)) < rel_err(Fr, D, slice(1, 4))


def test_1e10_exclusion_matches_mask_closely():
    s = small_system(400, 15.0, seed=5)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    R = oracle.field_direct(*args, 1)
    M = oracle.field_direct(*args, 1, excl_mode="mask")
    assert rel_err(R, M, slice(1, 4)) < 1e-14
    assert rel_err(R, M, slice(0, 1)) < 1e-8


def test_damped_far_limit_is_undamped():
    x, y, z = np.array([100.0]), np.array([80.0]), np.array([30.0])
    T0 = oracle.tensors(4, x, y, z, "", coef="exact")
    for d in ("THOLE", "ERF"):
        Td = oracle.tensors(4, x, y, z, d, [0.6], coef="exact")
        assert np.allclose(Td, T0, rtol=1e-12, atol=0)


def test_tree_invariants():
    from fmm_gb300 import systems
    X = systems.water(2000, 50.0, seed=6)["coordinates"]
    for cm in ("sequential", "blocked"):
        t = oracle.tree(X, 40, 0.5, centroid=cm)
        leaf = t["is_leaf"] == 1
        assert np.all(t["count"][leaf] < 40)
        assert np.all(t["count"][~leaf] >= 40)
        assert t["count"][leaf].sum() == X.shape[0]
        assert np.all(t["parent"][1:] < np.arange(1, len(t["parent"])))
        # every leaf near-list contains the leaf itself
        nl = set(map(tuple, t["near"]))
        for k in np.nonzero(leaf)[0]:
            assert (k, k) in nl

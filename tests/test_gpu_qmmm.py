"""QM/MM helpers on the GPU (get_boxes, get_multipoles,
interpolate_electron_fields; src/fmm.F90:1134-1336) against outputs of the
reference's own code (tests/golden/ref_fields.npz) and against the oracle."""
import os

import numpy as np
import pytest

import fmm_gb300
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fx():
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_fields.npz"))


def _leafwise_sorted(idx, X, ncrit, theta):
    """Near-field indices with each leaf's run sorted: the GPU lists a leaf's
    particles in ascending index, the reference in its insertion order."""
    t = oracle.tree(X, ncrit, theta)
    leaf = t["leaf_of"][idx - 1]
    out = idx.copy()
    s = 0
    while s < len(idx):
        e = s
        while e < len(idx) and leaf[e] == leaf[s]:
            e += 1
        out[s:e] = np.sort(idx[s:e])
        s = e
    return out


def test_gpu_get_boxes_matches_reference(fx):
    th, nc, p, f = fx["qmmm_cfg"]
    X = fx["qmmm_X"]
    idx, bc, bi = fmm_gb300.get_boxes(X, fx["qmmm_T"], th, int(nc), int(p))
    assert np.array_equal(idx, _leafwise_sorted(fx["qmmm_idx_near"], X, int(nc), th))
    assert np.array_equal(bc, fx["qmmm_box_coordinates"])
    assert np.array_equal(bi, fx["qmmm_box_indices"])


def test_gpu_get_multipoles_matches_reference(fx):
    th, nc, p, f = fx["qmmm_cfg"]
    X = fx["qmmm_X"]
    idx, bc, bm = fmm_gb300.get_multipoles(0, X, fx["qmmm_M"], fx["qmmm_T"], th, int(nc), int(p))
    assert np.array_equal(idx, _leafwise_sorted(fx["qmmm_idx_near_mp"], X, int(nc), th))
    assert np.array_equal(bc, fx["qmmm_box_coordinates_mp"])
    ref = fx["qmmm_box_multipoles"]
    assert bm.shape == ref.shape
    assert np.max(np.abs(bm - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_gpu_interpolate_electron_fields_matches_reference(fx):
    th, nc, p, f = fx["qmmm_cfg"]
    F = fmm_gb300.interpolate_electron_fields(0, fx["qmmm_X"], fx["qmmm_local"], fx["qmmm_box_indices"], th, int(nc),
                                              int(p), int(f))
    ref = fx["qmmm_field"]
    assert np.linalg.norm(F - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("ntgt,theta,p", [(1, 0.5, 6), (40, 0.4, 8), (300, 0.7, 5)])
def test_gpu_qmmm_helpers_match_oracle_larger(ntgt, theta, p):
    from fmm_gb300 import systems
    s = systems.water(4000, 50.0, seed=ntgt)
    X = s["coordinates"]
    rng = np.random.default_rng(ntgt)
    T = X[rng.choice(X.shape[0], ntgt, replace=False)] + rng.normal(0, 0.5, (ntgt, 3))
    M = np.stack([s["multipoles"], -0.3 * s["multipoles"]], axis=2)
    idx, bc, bi = fmm_gb300.get_boxes(X, T, theta, 32, p)
    oi, obc, obi = oracle.get_boxes(X, T, theta, 32, p)
    assert np.array_equal(idx, _leafwise_sorted(oi, X, 32, theta))
    assert np.array_equal(bc, obc) and np.array_equal(bi, obi)
    idx2, bc2, bm = fmm_gb300.get_multipoles(0, X, M, T, theta, 32, p)
    _, _, obm = oracle.get_multipoles(0, X, M, T, theta, 32, p)
    assert np.max(np.abs(bm - obm)) <= 1e-12 * np.max(np.abs(obm))
    nq = (p + 1) * (p + 2) * (p + 3) // 6
    Lx = rng.normal(0, 1.0, (len(bi), nq, 2)) / (1.0 + np.arange(nq))[None, :, None]
    F = fmm_gb300.interpolate_electron_fields(0, X, Lx, bi, theta, 32, p, 2)
    O = oracle.interpolate_electron_fields(0, X, Lx, bi, theta, 32, p, 2)
    assert np.linalg.norm(F - O) <= 1e-12 * np.linalg.norm(O)


def test_octree_module_exposes_the_helpers(fx):
    import octree
    th, nc, p, f = fx["qmmm_cfg"]
    a = octree.fmm.get_boxes(fx["qmmm_X"], fx["qmmm_T"], th, int(nc), int(p))
    b = fmm_gb300.get_boxes(fx["qmmm_X"], fx["qmmm_T"], th, int(nc), int(p))
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    F = octree.fmm.interpolate_electron_fields(0, fx["qmmm_X"], fx["qmmm_local"], fx["qmmm_box_indices"], th,
                                               int(nc), int(p), int(f))
    assert np.linalg.norm(F - fx["qmmm_field"]) <= 1e-12 * np.linalg.norm(fx["qmmm_field"])

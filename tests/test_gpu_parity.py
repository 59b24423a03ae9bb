"""GPU parity: the CUDA library against the CPU oracle on the same inputs.

Bars: bit-exact for the tree and lists (integer work); relative field error
<= 1e-12 for the FP64 paths (spec precision bar for the plain FP64
path).  Every call goes through the C ABI (include/fmm_gpu.h) via ctypes.
"""
import ctypes

import numpy as np
import pytest

import fmm_gb300
import oracle
from fmm_gb300 import Options, _lib
from helpers import rel_err, small_system

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _fmm_args(s):
    return (0, s["coordinates"], s["multipoles"], s["exclusions"])


@pytest.mark.parametrize("damp", ["", "THOLE", "AMOEBA", "ERF"])
@pytest.mark.parametrize("mf", [(0, 0), (0, 1), (1, 1), (2, 1), (2, 2), (1, 2), (3, 0), (3, 1), (0, 3), (2, 3),
                                (3, 3)])
@pytest.mark.parametrize("excl", ["ref", "mask"])
def test_direct_matches_oracle(damp, mf, excl):
    m, f = mf
    s = small_system(500, 18.0, order=m, seed=1, damp=damp)
    d = s["damping_factors"] if damp else None
    G = fmm_gb300.field_direct(*_fmm_args(s), f, damp, d, options=Options(excl_mode=excl))
    O = oracle.field_direct(*_fmm_args(s), f, damp, d, excl_mode=excl)
    cols = slice(1, None) if (damp == "AMOEBA" and f > 0) else slice(0, None)
    assert np.all(np.isfinite(G))
    assert rel_err(G, O, cols) <= TOL


def _gpu_tree(X, ncrit, theta, centroid):
    L = _lib.lib()
    X = np.asfortranarray(X)
    n = X.shape[0]
    sizes = np.zeros(4, dtype=np.int64)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    L.fmm_debug_tree.restype = ctypes.c_int
    L.fmm_debug_tree.argtypes = [ctypes.c_int64, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_double,
                                 ctypes.c_int, ctypes.POINTER(ctypes.c_int64)] + [ctypes.c_void_p] * 10
    st = L.fmm_debug_tree(n, dp(X), ncrit, theta, centroid, sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                          *([None] * 10))
    assert st == 0
    M, nf, nn, md = (int(v) for v in sizes)
    out = dict(center=np.zeros((M, 3)), r=np.zeros(M), rmax=np.zeros(M), depth=np.zeros(M, np.int32),
               parent=np.zeros(M, np.int32), is_leaf=np.zeros(M, np.int32), count=np.zeros(M, np.int32),
               leaf_of=np.zeros(n, np.int32), far=np.zeros((max(nf, 1), 2), np.int32),
               near=np.zeros((max(nn, 1), 2), np.int32))
    st = L.fmm_debug_tree(n, dp(X), ncrit, theta, centroid, sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                          dp(out["center"]), dp(out["r"]), dp(out["rmax"]), ip(out["depth"]), ip(out["parent"]),
                          ip(out["is_leaf"]), ip(out["count"]), ip(out["leaf_of"]), ip(out["far"]),
                          ip(out["near"]))
    assert st == 0
    out["far"] = out["far"][:nf]
    out["near"] = out["near"][:nn]
    out["max_depth"] = md
    return out


@pytest.mark.parametrize("centroid", ["sequential", "blocked"])
@pytest.mark.parametrize("case", ["uniform", "water", "blobs"])
def test_tree_and_lists_bit_exact(centroid, case):
    from fmm_gb300 import systems
    if case == "uniform":
        X = systems.uniform_triplets(4096, 40.0, seed=0)["coordinates"]
        ncrit, theta = 64, 0.5
    elif case == "water":
        X = systems.water(3000, 60.0, seed=2)["coordinates"]
        ncrit, theta = 64, 0.5
    else:
        X = systems.blobs(20000, n_blobs=8, box=200.0, seed=3)["coordinates"]
        ncrit, theta = 32, 0.4
    g = _gpu_tree(X, ncrit, theta, {"sequential": 0, "blocked": 1}[centroid])
    o = oracle.tree(X, ncrit, theta, centroid=centroid)
    assert g["center"].shape == o["center"].shape
    assert np.array_equal(g["center"], o["center"])
    assert np.array_equal(g["r"], o["r"])
    assert np.array_equal(g["rmax"], o["rmax"])
    for k in ("depth", "parent", "is_leaf", "count", "leaf_of"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["far"], o["far"])
    assert np.array_equal(g["near"], o["near"])


def test_fmm_ref_mode_matches_oracle_config1():
    """Config-1 shape: N=4096 uniform triplets, p=5, f=1, theta=0.5, ncrit=64."""
    from fmm_gb300 import systems
    s = systems.uniform_triplets(4096, 40.0, seed=0)
    G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 64, 5, 1)
    O = oracle.field_fmm(*_fmm_args(s), 0.5, 64, 5, 1)
    assert np.all(np.isfinite(G))
    assert rel_err(G, O) <= TOL


@pytest.mark.parametrize("damp,p,f", [("THOLE", 6, 2), ("AMOEBA", 8, 1), ("ERF", 4, 1), ("", 8, 2)])
def test_fmm_ref_mode_matches_oracle_damped(damp, p, f):
    """Reference semantics including the int32-wrapped Cnij table at p >= 6."""
    from fmm_gb300 import systems
    s = systems.water(800, 40.0, seed=4)
    if damp == "ERF":
        s["damping_factors"] = np.random.default_rng(5).uniform(0.3, 0.8, 2400)
    d = s["damping_factors"] if damp else None
    G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, p, f, damp, d)
    O = oracle.field_fmm(*_fmm_args(s), 0.5, 32, p, f, damp, d)
    cols = slice(1, None) if damp == "AMOEBA" else slice(0, None)
    assert rel_err(G, O, cols) <= TOL


@pytest.mark.parametrize("damp", ["", "THOLE", "AMOEBA", "ERF"])
@pytest.mark.parametrize("mf", [(3, 1), (2, 3), (3, 3)])
@pytest.mark.parametrize("coef", ["ref", "exact"])
def test_fmm_higher_orders_match_oracle(damp, mf, coef):
    """Octupole sources (mdim 20) and field order 3 (damped tensors up to
    order 6), FP64, both coefficient modes."""
    m, f = mf
    s = small_system(1500, 30.0, order=m, seed=31, damp=damp)
    d = s["damping_factors"] if damp else None
    if coef == "ref":
        G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 6, f, damp, d)
        O = oracle.field_fmm(*_fmm_args(s), 0.5, 32, 6, f, damp, d)
    else:
        G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 7, f, damp, d, options=Options.exact())
        O = oracle.field_fmm(*_fmm_args(s), 0.5, 32, 7, f, damp, d, coef_mode="exact", excl_mode="mask",
                             centroid_mode="blocked")
    cols = slice(1, None) if damp == "AMOEBA" else slice(0, None)
    assert np.all(np.isfinite(G[:, cols]))
    assert rel_err(G, O, cols) <= TOL


def test_higher_orders_refused_by_the_mixed_path():
    s = small_system(600, 20.0, order=3, seed=32)
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 6, 1, options=Options(precision="mixed"))
    s = small_system(600, 20.0, order=2, seed=32)
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 6, 3, options=Options(precision="mixed"))


@pytest.mark.parametrize("damp", ["", "THOLE"])
def test_fmm_exact_mode_matches_oracle(damp):
    from fmm_gb300 import systems
    s = systems.water(1200, 45.0, seed=6)
    d = s["damping_factors"] if damp else None
    opt = Options.exact()
    G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 6, 1, damp, d, options=opt)
    O = oracle.field_fmm(*_fmm_args(s), 0.5, 32, 6, 1, damp, d, coef_mode="exact", excl_mode="mask",
                         centroid_mode="blocked")
    assert rel_err(G, O) <= TOL


@pytest.mark.parametrize("p", [2, 9, 11, 12])
def test_fmm_exact_mode_all_orders(p):
    """Grouped reduced-basis M2L at low and high orders (FP64 products up to
    p = 11, the per-pair FP64 kernel at p = 12; FP32 products at all orders)."""
    from fmm_gb300 import systems
    s = systems.water(1200, 45.0, seed=16)
    O = oracle.field_fmm(*_fmm_args(s), 0.5, 32, p, 1, coef_mode="exact", excl_mode="mask", centroid_mode="blocked")
    G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, p, 1, options=Options.exact())
    assert rel_err(G, O) <= TOL
    Gm = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, p, 1, options=Options.exact(precision="mixed"))
    assert rel_err(Gm, O, slice(1, None)) < 5e-6


def test_theta_to_zero_is_direct():
    s = small_system(700, 20.0, seed=7)
    G = fmm_gb300.field_fmm(*_fmm_args(s), 1e-3, 16, 4, 1)
    D = fmm_gb300.field_direct(*_fmm_args(s), 1)
    assert rel_err(G, D) <= 1e-13


def test_small_n_falls_back_to_direct():
    s = small_system(50, 8.0, seed=8)
    G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 64, 5, 1)
    D = fmm_gb300.field_direct(*_fmm_args(s), 1)
    assert np.array_equal(G, D)


def test_exclusion_edge_cases():
    s = small_system(300, 12.0, seed=9)
    X, M = s["coordinates"], s["multipoles"]
    # no exclusion column at all: reference semantics give a non-finite self term
    E0 = np.zeros((300, 0), dtype=np.int32)
    F = fmm_gb300.field_direct(0, X, M, E0, 1)
    assert not np.all(np.isfinite(F))
    Fm = fmm_gb300.field_direct(0, X, M, E0, 1, options=Options(excl_mode="mask"))
    Om = oracle.field_direct(0, X, M, E0, 1, excl_mode="mask")
    assert rel_err(Fm, Om) <= TOL
    # duplicated and zero-padded entries behave like the set of listed partners
    E = np.asfortranarray(np.concatenate([s["exclusions"], s["exclusions"][:, :1], np.zeros((300, 1), np.int32)], 1))
    G = fmm_gb300.field_direct(0, X, M, E, 1)
    O = oracle.field_direct(0, X, M, E, 1)
    assert rel_err(G, O) <= TOL


def test_invalid_arguments_raise():
    s = small_system(100, 10.0, seed=10)
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 16, 4, 1, "BOGUS", None)
    bad = s["exclusions"].copy()
    bad[0, 0] = 101
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_direct(0, s["coordinates"], s["multipoles"], bad, 1)
    # periodic boxes need a box matrix and more than ncrit particles
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 16, 4, 1, "", None, True, None)
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 400, 4, 1, "", None, True, np.eye(3) * 10.0)


@pytest.mark.parametrize("damp", ["AMOEBA", "THOLE", "ERF"])
def test_damping_aware_acceptance_matches_oracle(damp):
    """mac_mode 'damping': far-field pairs closer than the damping range are
    demoted to the near field; same lists and fields as the oracle."""
    from fmm_gb300 import systems
    s = systems.water(1500, 50.0, seed=12)
    if damp == "ERF":
        s["damping_factors"] = np.random.default_rng(13).uniform(0.3, 0.8, 4500)
    d = s["damping_factors"]
    opt = Options.exact(mac_mode="damping")
    G = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 6, 1, damp, d, options=opt)
    O = oracle.field_fmm(*_fmm_args(s), 0.5, 32, 6, 1, damp, d, coef_mode="exact", excl_mode="mask",
                         centroid_mode="blocked", mac_mode="damping")
    assert rel_err(G, O) <= TOL
    st = fmm_gb300.last_stats()
    G0 = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 6, 1, damp, d, options=Options.exact())
    st0 = fmm_gb300.last_stats()
    assert st["p2p_particle_pairs"] > st0["p2p_particle_pairs"]
    D = fmm_gb300.field_direct(*_fmm_args(s), 1, damp, d, options=Options(excl_mode="mask"))
    assert rel_err(G, D, slice(1, 4)) < rel_err(G0, D, slice(1, 4))


@pytest.mark.parametrize("one_sided", [False, True])
def test_mixed_near_field_exclusions(one_sided):
    """The FP32 near field masks excluded partners by the target's own list,
    also when exclusions are listed by one partner only (the reference's
    per-target semantics); both match the FP64 path."""
    from fmm_gb300 import systems
    s = systems.water(4000, 70.0, order=2, seed=31)
    d = s["damping_factors"]
    E = np.array(s["exclusions"])
    if one_sided:
        E[1:600:3, :] = 0  # hydrogens of the first 200 molecules list nothing; their oxygens still do
    args = (0, s["coordinates"], s["multipoles"], np.asfortranarray(E))
    F64 = fmm_gb300.field_fmm(*args, 0.5, 64, 8, 1, "AMOEBA", d, options=Options.exact())
    F32 = fmm_gb300.field_fmm(*args, 0.5, 64, 8, 1, "AMOEBA", d, options=Options.exact(precision="mixed"))
    assert np.all(np.isfinite(F32))
    assert rel_err(F32, F64, slice(1, None)) < 5e-6


@pytest.mark.parametrize("p", [3, 10, 11, 12])
def test_m2l_tensor_core_product_matches_cuda_cores(p, monkeypatch):
    """The FP32 M2L product on the tensor cores (operands split into TF32
    parts, three products per term, FP32 accumulation in tensor memory) agrees
    with the same product on the CUDA cores and with the FP64 path."""
    from fmm_gb300 import systems
    s = systems.water(4000, 70.0, order=2, seed=21)
    d = s["damping_factors"]
    mixed = Options.exact(precision="mixed")
    F64 = fmm_gb300.field_fmm(*_fmm_args(s), 0.4, 64, p, 1, "AMOEBA", d, options=Options.exact())
    Ftc = fmm_gb300.field_fmm(*_fmm_args(s), 0.4, 64, p, 1, "AMOEBA", d, options=mixed)
    assert fmm_gb300.last_stats()["m2l_pairs"] > 0
    monkeypatch.setenv("FMM_GB300_M2L_PRODUCT", "cuda")
    Fcc = fmm_gb300.field_fmm(*_fmm_args(s), 0.4, 64, p, 1, "AMOEBA", d, options=mixed)
    assert np.all(np.isfinite(Ftc))
    assert rel_err(Ftc, Fcc, slice(1, None)) < 2e-6
    assert rel_err(Ftc, F64, slice(1, None)) < 5e-6


@pytest.mark.parametrize("scale", [1e-24, 1e-9, 1e20])
def test_mixed_precision_multipole_scale(scale):
    """The mixed path splits FP64 moments into FP32 pairs from their bit
    patterns (P2M, M2M, L2L): multipoles far from unit magnitude keep the
    accuracy of the unit-scale case (the field is linear in them)."""
    from fmm_gb300 import systems
    s = systems.water(4000, 70.0, order=2, seed=23)
    s["multipoles"] = s["multipoles"] * scale
    d = s["damping_factors"]
    F64 = fmm_gb300.field_fmm(*_fmm_args(s), 0.4, 64, 10, 1, "AMOEBA", d, options=Options.exact())
    F32 = fmm_gb300.field_fmm(*_fmm_args(s), 0.4, 64, 10, 1, "AMOEBA", d, options=Options.exact(precision="mixed"))
    assert np.all(np.isfinite(F32))
    assert rel_err(F32, F64, slice(1, None)) < 5e-6


@pytest.mark.parametrize("damp,mf", [("AMOEBA", (2, 1)), ("", (2, 2)), ("ERF", (1, 1)), ("THOLE", (0, 1))])
def test_mixed_precision_close_to_fp64(damp, mf):
    """FP32 near field and M2L with FP64 sums: within FP32 accuracy of the FP64
    path on the same tree and lists."""
    from fmm_gb300 import systems
    m, f = mf
    s = systems.water(4000, 70.0, order=m, seed=14)
    if damp == "ERF":
        s["damping_factors"] = np.random.default_rng(15).uniform(0.3, 0.8, 12000)
    d = s["damping_factors"] if damp else None
    F64 = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 64, 8, f, damp, d, options=Options.exact())
    F32 = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 64, 8, f, damp, d, options=Options.exact(precision="mixed"))
    assert np.all(np.isfinite(F32))
    # field columns (order >= 1); the potential column of a neutral system is a
    # sum with heavy cancellation and is not part of the accuracy target.  The
    # bound is the FP32 floor of a system of neutral groups of large charges
    # (per-pair rounding ~1e-7, amplified by the cancellation inside groups).
    assert rel_err(F32, F64, slice(1, None)) < 5e-6


@pytest.mark.parametrize("damp,mf", [("AMOEBA", (2, 1)), ("THOLE", (2, 1)), ("ERF", (1, 1)), ("", (2, 1)),
                                     ("AMOEBA", (0, 1)), ("THOLE", (1, 0))])
@pytest.mark.parametrize("one_sided", [False, True])
def test_packed_near_field_matches_one_source_kernel(damp, mf, one_sided, monkeypatch):
    """The packed near field (two sources per thread in f32x2 arithmetic, odd
    leaves padded with an empty particle, skipped halves zeroed) agrees with
    the one-source FP32 kernel to FP32 rounding, and both with the FP64 path;
    exclusions listed by one partner only included.  (erf damping runs the
    one-source kernel either way; its case checks that selection.)"""
    from fmm_gb300 import systems
    m, f = mf
    s = systems.water(3001, 70.0, order=m, seed=41)
    if damp == "ERF":
        s["damping_factors"] = np.random.default_rng(42).uniform(0.3, 0.8, 9003)
    d = s["damping_factors"] if damp else None
    E = np.array(s["exclusions"])
    if one_sided:
        E[1:900:3, :] = 0
    args = (0, s["coordinates"], s["multipoles"], np.asfortranarray(E))
    mixed = Options.exact(precision="mixed")
    F64 = fmm_gb300.field_fmm(*args, 0.5, 64, 8, f, damp, d, options=Options.exact())
    Fx2 = fmm_gb300.field_fmm(*args, 0.5, 64, 8, f, damp, d, options=mixed)
    monkeypatch.setenv("FMM_GB300_P2P_PACKED", "0")
    F1 = fmm_gb300.field_fmm(*args, 0.5, 64, 8, f, damp, d, options=mixed)
    assert np.all(np.isfinite(Fx2))
    if f > 0:
        assert rel_err(Fx2, F1, slice(1, None)) < 1e-6
        assert rel_err(Fx2, F64, slice(1, None)) < 5e-6
    else:
        # the potential of neutral groups: a sum with heavy cancellation
        assert rel_err(Fx2, F1) < 1e-5
        assert rel_err(Fx2, F64) < 5e-5


def test_release_workspace_then_call_again():
    """fmm_release_workspace frees the thread's device buffers; the next call
    allocates again and gives the same field."""
    s = small_system(900, 22.0, seed=7)
    F1 = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 5, 1)
    fmm_gb300.release_workspace()
    F2 = fmm_gb300.field_fmm(*_fmm_args(s), 0.5, 32, 5, 1)
    assert rel_err(F2, F1) <= 1e-14
    fmm_gb300.release_workspace()
    fmm_gb300.release_workspace()  # releasing an empty workspace is fine

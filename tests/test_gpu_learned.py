"""Learned expansion-order selector at run time on the GPU: the shipped
network meets the accuracy target, does less M2L work than the fixed rule,
follows the requested target, and a network that under-predicts errors is
caught by the sampled check (fixed-rule fallback)."""
import numpy as np
import pytest

import fmm_gb300
from fmm_gb300 import Options, systems
from helpers import per_target_rel

pytestmark = pytest.mark.gpu

N_MOL = 20000
BOX = 270.0 * (N_MOL / 333333.0) ** (1.0 / 3.0)  # density of the 1M-particle water workload


@pytest.fixture(scope="module")
def water():
    s = systems.water(N_MOL, BOX, order=2, seed=11)
    D = fmm_gb300.field_direct(0, s["coordinates"], s["multipoles"], s["exclusions"], 1, "AMOEBA",
                               s["damping_factors"], options=Options(excl_mode="mask"))
    return s, D


def _run(s, selector, **kw):
    opt = Options.exact(precision="mixed", mac_mode="damping", selector=selector, **kw)
    F = fmm_gb300.field_fmm(0, s["coordinates"], s["multipoles"], s["exclusions"], 0.3, 64, 10, 1, "AMOEBA",
                            s["damping_factors"], options=opt)
    return F, fmm_gb300.last_stats()


def _rms(F, D):
    e = per_target_rel(F, D, slice(1, 4))
    return float(np.sqrt(np.mean(e ** 2)))


def _m2l_work(st):
    return sum(st["m2l_pairs_q%d" % q] * (q + 1) ** 4 for q in range(13))


def test_learned_meets_target(water):
    s, D = water
    F, st = _run(s, "learned", target_rel_err=1e-6)
    assert st["selector_fallback"] == 0
    assert 0.0 <= st["sampled_rms_err"] <= 1e-6
    assert _rms(F, D) <= 1e-6


def test_learned_cheaper_than_fixed(water):
    s, D = water
    _, sf = _run(s, "fixed")
    _, sl = _run(s, "learned")
    assert sf["m2l_order_mean"] == 10.0
    assert sl["m2l_order_mean"] < 10.0
    assert _m2l_work(sl) < 0.8 * _m2l_work(sf)


def test_looser_target_lowers_orders(water):
    s, D = water
    Fa, a = _run(s, "learned", target_rel_err=1e-5)
    _, b = _run(s, "learned", target_rel_err=1e-6)
    assert a["m2l_order_mean"] < b["m2l_order_mean"]
    assert _rms(Fa, D) <= 1e-5


def test_underestimating_network_falls_back(water, tmp_path):
    s, D = water
    w = np.fromfile(fmm_gb300.SELECTOR_WEIGHTS, dtype="<f4").copy()
    # last layer: zero weights, bias -30 (predicts 1e-30 at every order, so
    # every accepted pair would get order 2)
    nout, nh = 11, 64
    w[-nout:] = -30.0
    w[-nout - nout * nh:-nout] = 0.0
    bad = tmp_path / "bad.bin"
    w.tofile(bad)
    fmm_gb300.load_selector(str(bad))
    try:
        F, st = _run(s, "learned")
    finally:
        fmm_gb300.load_selector()
    assert st["selector_fallback"] == 1
    assert st["m2l_order_mean"] == 10.0
    assert _rms(F, D) <= 1e-6


def test_learned_on_clustered_particles_meets_target():
    """Heterogeneous density (Gaussian blobs, the clustered benchmark system's
    kind at 120k particles): whichever path the call takes (the learned lists
    with per-node error budgets from the local field, or the fixed rule after
    a failed sampled check), the result meets the target at 256 sampled
    particles."""
    import bench
    sc = (120_000 / 2_000_000) ** (1.0 / 3.0)
    for seed in (5, 7):
        s = systems.blobs(n=120_000, box=600.0 * sc, sigma_range=(5.0 * sc, 30.0 * sc), seed=seed)
        opt = Options.exact(precision="mixed", mac_mode="damping", selector="learned")
        F = fmm_gb300.field_fmm(0, s["coordinates"], s["multipoles"], s["exclusions"], 0.3, 64, 12, 1, "AMOEBA",
                                s["damping_factors"], options=opt)
        rng = np.random.default_rng(1)
        rows = np.sort(rng.choice(F.shape[0], 256, replace=False))
        ref = bench.sampled_reference(s, rows, "AMOEBA")
        assert bench.rel_errors(F[rows], ref)["rms_rel_err"] <= 1e-6


def test_damping_correction_meets_target_with_fewer_near_pairs(water, monkeypatch):
    """Learned lists with the damping correction (leaf pairs inside the
    damping range accepted as far pairs, the damped-minus-undamped kernel of
    their close particle pairs added in the near field) meet the target like
    the demoting rule (FMM_GB300_DAMP_CORR=0) with fewer near pairs."""
    s, D = water
    F, st = _run(s, "learned")
    monkeypatch.setenv("FMM_GB300_DAMP_CORR", "0")
    F0, st0 = _run(s, "learned")
    assert st["selector_fallback"] == 0 and st0["selector_fallback"] == 0
    assert _rms(F, D) <= 1e-6
    assert _rms(F0, D) <= 1e-6
    assert st["p2p_particle_pairs"] < st0["p2p_particle_pairs"]
    assert st["corr_leaf_pairs"] > 0
    assert st0["corr_leaf_pairs"] == 0 and st0["corr_particle_pairs"] == 0


def test_damping_correction_with_distant_exclusions(water):
    """Exclusions between particles of distant leaves: an excluded pair in a
    corrected far leaf pair gets neither the correction nor the field (the
    M2L's undamped share is removed by the exclusion pass), as in the direct
    sum; the result meets the target (with the learned lists or, when the
    sampled check rejects them, with the fixed rule)."""
    s, _ = water
    n = s["coordinates"].shape[0]
    E = np.hstack([np.array(s["exclusions"]), np.zeros((n, 1), dtype=np.array(s["exclusions"]).dtype)])
    rng = np.random.default_rng(13)
    # 600 pairs of particles 10-14 bohr apart also exclude each other (both lists)
    X = s["coordinates"]
    picked = 0
    for i in rng.permutation(n):
        if picked >= 600:
            break
        if E[i, -1] != 0:
            continue
        d = np.linalg.norm(X - X[i], axis=1)
        cand = [j for j in np.nonzero((d > 10.0) & (d < 14.0))[0] if E[j, -1] == 0]
        if not cand:
            continue
        j = int(cand[0])
        E[i, -1] = j + 1
        E[j, -1] = i + 1
        picked += 1
    assert picked == 600
    E2 = np.asfortranarray(E)
    D = fmm_gb300.field_direct(0, X, s["multipoles"], E2, 1, "AMOEBA", s["damping_factors"],
                               options=Options(excl_mode="mask"))
    opt = Options.exact(precision="mixed", mac_mode="damping", selector="learned")
    F = fmm_gb300.field_fmm(0, X, s["multipoles"], E2, 0.3, 64, 10, 1, "AMOEBA", s["damping_factors"], options=opt)
    st = fmm_gb300.last_stats()
    if st["selector_fallback"] == 0:
        assert st["corr_leaf_pairs"] > 0
    assert _rms(F, D) <= 1e-6


def test_damping_correction_applied_with_longer_damping_range(water):
    """Damping factors scaled by 0.7 (a longer damping range): the learned
    lists' far leaf pairs inside the range hold millions of particle pairs
    whose damping correction is evaluated; the result stays at the FP32
    floor of such a strongly damped system (about 1.2e-6 for the fixed rule
    on the same mixed path, measured), where a wrong correction would be
    orders of magnitude off."""
    s, _ = water
    d = s["damping_factors"] * 0.7
    D = fmm_gb300.field_direct(0, s["coordinates"], s["multipoles"], s["exclusions"], 1, "AMOEBA", d,
                               options=Options(excl_mode="mask"))
    opt = Options.exact(precision="mixed", mac_mode="damping", selector="learned")
    F = fmm_gb300.field_fmm(0, s["coordinates"], s["multipoles"], s["exclusions"], 0.3, 64, 10, 1, "AMOEBA", d,
                            options=opt)
    st = fmm_gb300.last_stats()
    if st["selector_fallback"] == 0:
        assert st["corr_particle_pairs"] > 1e6
    assert _rms(F, D) <= 2e-6

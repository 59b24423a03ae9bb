"""The mixed-precision near field's launch shapes (threads per block, staging
size, cost-ordered work queue) and the autotuner that picks ncrit and the
shape per class of calls."""
import os

import numpy as np
import pytest

import fmm_gb300
from fmm_gb300 import Options, systems
from helpers import rel_err

pytestmark = pytest.mark.gpu

MIXED = Options(precision="mixed", mac_mode="damping")


@pytest.fixture(scope="module")
def water():
    return systems.water(20_000, 270.0 * (20_000 / 333_333) ** (1 / 3), seed=51)


def _fmm(s, opt, ncrit=64):
    return fmm_gb300.field_fmm(0, s["coordinates"], s["multipoles"], s["exclusions"], 0.3, ncrit, 8, 1, "AMOEBA",
                               s["damping_factors"], options=opt)


def test_near_field_shapes_agree(water):
    F0 = _fmm(water, MIXED)
    try:
        # same staging size: the same sums in the same order
        for sh in [(128, 320, 0), (256, 320, 0), (256, 320, 1), (64, 320, 1)]:
            fmm_gb300.set_p2p_shape(*sh)
            F = _fmm(water, MIXED)
            st = fmm_gb300.last_stats()
            assert (st["p2p_threads"], st["p2p_stage"], st["p2p_queue"]) == sh
            assert np.array_equal(F, F0), sh
        # other staging sizes regroup the compensated per-piece sums
        for sh in [(128, 160, 0), (128, 640, 1), (64, 1024, 0), (256, 64, 1)]:
            fmm_gb300.set_p2p_shape(*sh)
            F = _fmm(water, MIXED)
            assert rel_err(F, F0, slice(1, None)) <= 1e-7, sh
    finally:
        fmm_gb300.set_p2p_shape()
    assert fmm_gb300.last_stats()["p2p_stage"] > 0


def test_set_p2p_shape_rejects_bad_shapes():
    for sh in [(100, 320, 0), (128, 8, 0), (128, 330, 0), (128, 320, 2), (512, 320, 0)]:
        with pytest.raises(fmm_gb300.FmmError):
            fmm_gb300.set_p2p_shape(*sh)


def test_autotune_tunes_once_per_class(water, tmp_path, monkeypatch):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("FMM_GB300_TUNE_CACHE", str(cache))
    opt = Options(precision="mixed", mac_mode="damping", autotune=True)
    F1 = _fmm(water, opt, ncrit=40)
    st1 = fmm_gb300.last_stats()
    F2 = _fmm(water, opt, ncrit=40)
    st2 = fmm_gb300.last_stats()
    assert st1["tuned"] == 1 and st2["tuned"] == 0
    for k in ("ncrit_used", "p2p_threads", "p2p_stage", "p2p_queue"):
        assert st1[k] == st2[k]
    assert st1["ncrit_used"] in (32, 40, 48, 64, 96, 128)
    assert np.array_equal(F1, F2)
    # accuracy at sampled particles against the FP64 direct sum
    rng = np.random.default_rng(3)
    rows = np.sort(rng.choice(F1.shape[0], 48, replace=False))
    D = fmm_gb300.field_direct(0, water["coordinates"], water["multipoles"], water["exclusions"], 1, "AMOEBA",
                               water["damping_factors"], options=Options(excl_mode="mask"))
    assert rel_err(F1[rows], D[rows], slice(1, None)) <= 1e-5
    # untuned calls keep the default shape
    _fmm(water, MIXED)
    st3 = fmm_gb300.last_stats()
    assert (st3["p2p_threads"], st3["p2p_stage"], st3["p2p_queue"], st3["tuned"]) == (128, 320, 1, 0)
    lines = [l.split() for l in open(cache).read().splitlines() if l.strip()]
    if lines:  # the cache file is read once per process (it may be another test's)
        assert all(len(l) == 5 for l in lines)


def test_autotune_batched_systems():
    rng = np.random.default_rng(7)
    sys_list = [systems.water(int(k), 12.0 * (k / 300.0) ** (1 / 3), seed=60 + i)
                for i, k in enumerate(rng.integers(300, 3000, 40))]
    opt = Options(precision="mixed", mac_mode="damping", autotune=True)
    G = fmm_gb300.field_fmm_batched(sys_list, 0.5, 32, 6, 1, "AMOEBA", options=opt)
    assert fmm_gb300.last_stats()["tuned"] == 1
    H = fmm_gb300.field_fmm_batched(sys_list, 0.5, 32, 6, 1, "AMOEBA", options=MIXED)
    for g, h in zip(G, H):
        assert rel_err(g, h, slice(1, None)) <= 1e-4


def test_autotune_refused_where_it_does_not_apply(water):
    opt = Options(precision="mixed", autotune=True)
    s = systems.water(200, 15.0, seed=52)
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_fmm(0, s["coordinates"], s["multipoles"], s["exclusions"], 0.5, 16, 4, 1, "", None, True,
                            np.eye(3) * 15.0, options=Options(autotune=True))
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.Plan(s["coordinates"], 10, s["exclusions"], 0.5, 16, 4, 1, options=opt)

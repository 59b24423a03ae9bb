"""Batched independent systems (fmm_field_fmm_batched) on the GPU."""
import numpy as np
import pytest

import fmm_gb300
from fmm_gb300 import Options, systems
from helpers import rel_err

pytestmark = pytest.mark.gpu


def _systems(k=7, seed=5):
    sl = systems.batched_uniform(n_systems=k, nmin=400, nmax=4000, density=0.1, order=1, seed=seed)
    return sl


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_matches_direct_per_system(precision):
    sl = _systems()
    opt = Options.exact(precision=precision)
    Fb = fmm_gb300.field_fmm_batched(sl, 0.3, 32, 10, 1, "ERF", options=opt)
    # truncation error of these settings is ~5e-8 (CPU oracle, same systems);
    # the FP32 near field adds ~6e-7 for erf damping
    tol = 1e-6 if precision == "fp64" else 5e-6
    for s, F in zip(sl, Fb):
        D = fmm_gb300.field_direct(0, s["coordinates"], s["multipoles"], s["exclusions"], 1, "ERF",
                                   s["damping_factors"], options=Options(excl_mode="mask"))
        assert rel_err(F, D, slice(1, 4)) < tol


def test_batched_agrees_with_separate_calls():
    sl = _systems(k=5, seed=6)
    opt = Options.exact()
    Fb = fmm_gb300.field_fmm_batched(sl, 0.3, 32, 10, 1, "ERF", options=opt)
    for s, F in zip(sl, Fb):
        G = fmm_gb300.field_fmm(0, s["coordinates"], s["multipoles"], s["exclusions"], 0.3, 32, 10, 1, "ERF",
                                s["damping_factors"], options=opt)
        # the packed tree differs from the single-system tree, so the two
        # agree to the truncation error of the settings (~5e-8)
        assert rel_err(F, G, slice(1, 4)) < 1e-6


def test_no_crosstalk_between_systems():
    sl = _systems(k=6, seed=7)
    opt = Options.exact()
    F1 = fmm_gb300.field_fmm_batched(sl, 0.5, 32, 6, 1, "ERF", options=opt)
    sl2 = [dict(s) for s in sl]
    sl2[2] = dict(sl[2])
    sl2[2]["multipoles"] = np.asfortranarray(sl[2]["multipoles"] * 3.0 + 0.1)
    F2 = fmm_gb300.field_fmm_batched(sl2, 0.5, 32, 6, 1, "ERF", options=opt)
    for k in range(len(sl)):
        if k == 2:
            assert not np.array_equal(F1[k], F2[k])
        else:
            assert np.array_equal(F1[k], F2[k]), k


def test_batched_rejects_tiny_systems():
    sl = _systems(k=3, seed=8)
    sl[1] = {key: (v[:20] if hasattr(v, "shape") else v) for key, v in sl[1].items()}
    sl[1]["exclusions"] = np.arange(1, 21, dtype=np.int32).reshape(20, 1)
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.field_fmm_batched(sl, 0.5, 32, 6, 1, "ERF", options=Options.exact())

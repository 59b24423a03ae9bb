"""Plans: fixed coordinates, many multipole sets, each evaluation one CUDA
graph launch.  Every evaluation must give what field_fmm gives for the same
inputs (which the parity tests pin to the oracle), in every precision mode."""
import numpy as np
import pytest

import fmm_gb300
import oracle
from fmm_gb300 import Options, systems
from helpers import rel_err

pytestmark = pytest.mark.gpu


def _sets(s, k, seed):
    rng = np.random.default_rng(seed)
    M0 = np.asarray(s["multipoles"])
    return [np.asfortranarray(M0 * rng.uniform(0.5, 1.5) + rng.normal(0, 0.02, M0.shape)) for _ in range(k)]


@pytest.mark.parametrize("damp,opt,tol", [("", None, 1e-14), ("AMOEBA", None, 1e-14),
                                          ("THOLE", Options.exact(), 1e-14),
                                          ("AMOEBA", Options(precision="mixed", mac_mode="damping"), 1e-13)])
def test_plan_matches_field_fmm(damp, opt, tol):
    s = systems.water(3000, 45.0, seed=41)
    d = s["damping_factors"] if damp else None
    X, E = s["coordinates"], s["exclusions"]
    with fmm_gb300.Plan(X, 10, E, 0.5, 32, 6, 1, damp, d, options=opt) as plan:
        assert plan.kernels > 5
        for M in _sets(s, 3, 1):
            F = plan.execute(M)
            G = fmm_gb300.field_fmm(0, X, M, E, 0.5, 32, 6, 1, damp, d, options=opt)
            cols = slice(1, None) if damp == "AMOEBA" else slice(0, None)
            assert np.all(np.isfinite(F[:, cols]))
            assert rel_err(F, G, cols) <= tol


def test_plan_matches_oracle_and_is_linear():
    s = systems.water(2000, 40.0, seed=42)
    X, E = s["coordinates"], s["exclusions"]
    M1, M2 = _sets(s, 2, 2)
    with fmm_gb300.Plan(X, 10, E, 0.5, 32, 5, 2, options=Options.exact()) as plan:
        F1 = plan.execute(M1)
        F2 = plan.execute(M2)
        F3 = plan.execute(np.asfortranarray(0.3 * M1 - 1.7 * M2))
    O1 = oracle.field_fmm(0, X, M1, E, 0.5, 32, 5, 2, coef_mode="exact", excl_mode="mask", centroid_mode="blocked")
    assert rel_err(F1, O1) <= 1e-12
    assert rel_err(F3, 0.3 * F1 - 1.7 * F2) <= 1e-12


def test_plan_small_system_is_direct_sum():
    s = systems.water(10, 8.0, seed=43)
    X, E = s["coordinates"], s["exclusions"]
    M = _sets(s, 1, 3)[0]
    with fmm_gb300.Plan(X, 10, E, 0.5, 64, 5, 1) as plan:
        F = plan.execute(M)
    D = fmm_gb300.field_direct(0, X, M, E, 1)
    assert rel_err(F, D) <= 1e-14


def test_plan_independent_of_other_calls_and_device_arrays():
    torch = pytest.importorskip("torch")
    s = systems.water(2500, 42.0, seed=44)
    X, E = s["coordinates"], s["exclusions"]
    M1, M2 = _sets(s, 2, 4)
    plan = fmm_gb300.Plan(X, 10, E, 0.5, 32, 6, 1)
    F1 = plan.execute(M1)
    # other calls on the thread's own workspace (another size) in between
    o = systems.water(5000, 55.0, seed=45)
    fmm_gb300.field_fmm(0, o["coordinates"], o["multipoles"], o["exclusions"], 0.5, 32, 8, 2)
    F1b = plan.execute(M1)
    assert np.array_equal(F1, F1b)
    dM = torch.tensor(np.asarray(M2).T.copy(), dtype=torch.float64, device="cuda").T
    dF = torch.zeros((4, X.shape[0]), dtype=torch.float64, device="cuda").T
    plan.execute_device(dM, dF)
    torch.cuda.synchronize()
    assert rel_err(dF.cpu().numpy(), plan.execute(M2)) <= 1e-15
    plan.close()


def test_plan_argument_checks():
    s = systems.water(500, 25.0, seed=46)
    X, E = s["coordinates"], s["exclusions"]
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.Plan(X, 10, E, 0.5, 32, 10, 1, "AMOEBA", s["damping_factors"],
                       options=Options(precision="mixed", selector="learned"))
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.Plan(X, 20, E, 0.5, 32, 6, 1, options=Options(precision="mixed"))
    with pytest.raises(fmm_gb300.FmmError):
        fmm_gb300.Plan(X, 7, E, 0.5, 32, 6, 1)
    with fmm_gb300.Plan(X, 10, E, 0.5, 32, 6, 1) as plan:
        with pytest.raises(ValueError):
            plan.execute(np.zeros((X.shape[0], 4)))


@pytest.mark.parametrize("opt", [Options.exact(), Options.exact(precision="mixed")])
def test_batched_plan_matches_batched_call(opt):
    sl = systems.batched_uniform(n_systems=9, nmin=400, nmax=4000, density=0.1, order=1, seed=8)
    Fb = fmm_gb300.field_fmm_batched(sl, 0.5, 32, 6, 1, "ERF", options=opt)
    with fmm_gb300.Plan.batched(sl, 4, 0.5, 32, 6, 1, "ERF", options=opt) as plan:
        Fp = plan.execute_systems([s["multipoles"] for s in sl])
        Fp2 = plan.execute_systems([2.0 * np.asarray(s["multipoles"]) for s in sl])
    for a, b, c in zip(Fb, Fp, Fp2):
        assert rel_err(b, a) <= 1e-13
        assert rel_err(c, 2.0 * a) <= 1e-12

"""Full-size benchmark configurations in reference mode against the oracle.

* The Thole water system of N = 199,998 (66,666 triplets in a 125 bohr cube,
  multipoles of order 2, theta 0.5, ncrit 64, expansion order 6, field
  order 2): every particle, relative field error <= 1e-12.
* The AMOEBA water system of N = 999,999 (333,333 triplets in a 270 bohr
  cube, theta 0.5, ncrit 64, expansion order 8, field order 1): on 8,192
  random particles and on all of them, field columns (AMOEBA has no
  potential).
Both use the reference's semantics (int32 Cnij closed form, excluded
sources at 1e10, reference acceptance rule), so the expected values are the
reference's own, defects included (src/fmm.F90:1354-1400).  The oracle runs
on all host cores and takes tens of seconds at these sizes.
"""
import numpy as np
import pytest

import fmm_gb300
import oracle
from fmm_gb300 import systems
from helpers import rel_err

pytestmark = pytest.mark.gpu


def test_thole_water_200k_ref_mode():
    s = systems.water(66_666, 125.0, seed=2)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    G = fmm_gb300.field_fmm(*args, 0.5, 64, 6, 2, "THOLE", s["damping_factors"])
    O = oracle.field_fmm(*args, 0.5, 64, 6, 2, "THOLE", s["damping_factors"])
    assert G.shape == (199_998, 10)
    assert np.all(np.isfinite(G))
    assert rel_err(G, O) <= 1e-12
    assert rel_err(G, O, slice(1, 4)) <= 1e-12


def test_amoeba_water_1m_ref_mode_sampled():
    s = systems.water(333_333, 270.0, seed=3)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    G = fmm_gb300.field_fmm(*args, 0.5, 64, 8, 1, "AMOEBA", s["damping_factors"])
    O = oracle.field_fmm(*args, 0.5, 64, 8, 1, "AMOEBA", s["damping_factors"])
    rng = np.random.default_rng(8192)
    tgt = np.sort(rng.choice(G.shape[0], 8192, replace=False))
    assert np.all(np.isfinite(G[tgt]))
    assert rel_err(G[tgt], O[tgt], slice(1, 4)) <= 1e-12
    assert rel_err(G, O, slice(1, 4)) <= 1e-12

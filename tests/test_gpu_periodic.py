"""Periodic cells on the GPU (src/fmm.F90:156-175, 337-343, 623-979): the
CUDA library against the CPU oracle in both coefficient and exclusion modes,
the lattice-sum bookkeeping, and the argument checks.  The reference's own
periodic outputs are checked in test_gpu_ref_golden.py."""
import numpy as np
import pytest

import fmm_gb300
import oracle
from fmm_gb300 import Options, _lib
from helpers import potential_up_to_constant, rel_err

pytestmark = pytest.mark.gpu


def _cell_system(n_mol, H, seed, order=2):
    from fmm_gb300 import systems
    s = systems.water(n_mol, float(np.max(H)), order=order, seed=seed)
    u = np.mod(np.linalg.solve(H, np.asarray(s["coordinates"]).T).T, 1.0)
    s["coordinates"] = np.asfortranarray(u @ H.T)
    return s


TRICLINIC = np.array([[22.0, 0.0, 0.0], [3.0, 21.0, 0.0], [-2.0, 1.5, 20.0]]).T  # cell vectors as columns
CUBIC = np.diag([22.0, 22.0, 22.0])


@pytest.mark.parametrize("damp,p,f,cell", [("", 5, 1, "triclinic"), ("THOLE", 6, 2, "triclinic"),
                                           ("ERF", 4, 1, "triclinic"), ("", 6, 1, "cubic"),
                                           ("AMOEBA", 5, 2, "cubic")])
@pytest.mark.parametrize("mode", ["ref", "exact"])
def test_periodic_matches_oracle(damp, p, f, cell, mode):
    """Field columns to 1e-12.  The potential column to 1e-12 up to a
    constant, and in full where the lattice sum converged (the reference's
    convergence test never passes for these triclinic cells; after its 50
    levels the potential's constant is dominated by rounding)."""
    H = TRICLINIC if cell == "triclinic" else CUBIC
    s = _cell_system(200, H, seed=31)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    d = s["damping_factors"] if damp else None
    box = np.asfortranarray(H)
    if mode == "ref":
        G = fmm_gb300.field_fmm(*args, 0.5, 24, p, f, damp, d, True, box)
        O = oracle.field_fmm(*args, 0.5, 24, p, f, damp, d, True, box)
    else:
        G = fmm_gb300.field_fmm(*args, 0.5, 24, p, f, damp, d, True, box,
                                options=Options(coef_mode="exact", excl_mode="mask"))
        O = oracle.field_fmm(*args, 0.5, 24, p, f, damp, d, True, box, coef_mode="exact", excl_mode="mask")
    assert np.all(np.isfinite(G))
    assert rel_err(G, O, slice(1, None)) <= 1e-12
    st = fmm_gb300.last_stats()
    levels = st["lattice_levels"]
    assert levels == oracle.last_lattice_levels()
    # far pairs of all 27 images, counted by expansion order image by image
    assert sum(st["m2l_pairs_q%d" % q] for q in range(13)) == st["m2l_pairs"] > 0
    var, const = potential_up_to_constant(G, O)
    assert var <= 1e-12
    if levels < 50:
        assert rel_err(G, O, slice(0, 1)) <= 1e-12


def test_periodic_differs_from_open_boundaries():
    """The images and the lattice contribute: the periodic field is not the
    open-boundary field of the same particles."""
    s = _cell_system(150, CUBIC, seed=32)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    box = np.asfortranarray(CUBIC)
    Gp = fmm_gb300.field_fmm(*args, 0.5, 24, 5, 1, "", None, True, box)
    assert fmm_gb300.last_stats()["lattice_levels"] >= 1
    Go = fmm_gb300.field_fmm(*args, 0.5, 24, 5, 1)
    assert rel_err(Gp, Go, slice(1, 4)) > 1e-3
    assert fmm_gb300.last_stats()["lattice_levels"] == 0


def test_periodic_argument_checks():
    s = _cell_system(40, TRICLINIC, seed=33)
    args = (0, s["coordinates"], s["multipoles"], s["exclusions"])
    box = np.asfortranarray(TRICLINIC)
    with pytest.raises(fmm_gb300.FmmError) as e:
        fmm_gb300.field_fmm(*args, 0.5, 16, 5, 1, "", None, True, None)  # no box
    assert e.value.status == _lib.FMM_EINVAL
    with pytest.raises(fmm_gb300.FmmError) as e:
        fmm_gb300.field_fmm(*args, 0.5, 500, 5, 1, "", None, True, box)  # n <= ncrit
    assert e.value.status == _lib.FMM_EINVAL
    with pytest.raises(fmm_gb300.FmmError) as e:
        fmm_gb300.field_fmm(*args, 0.5, 16, 5, 1, "", None, True, box, options=Options.exact(precision="mixed"))
    assert e.value.status == _lib.FMM_ENOTSUP

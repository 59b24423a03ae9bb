"""The CPU oracle against outputs of the reference's own source code.

The fixtures in tests/golden/ref_*.npz were produced by executing the
reference's Fortran statements (src/fmm.F90, src/tensors*.F90) through a
mechanical translation (tests/golden/fortran_exec.py, driven by
tests/golden/make_ref_golden.py).  These tests pin the oracle to them:
integer tables and the octree/interaction lists bit for bit, tensors and
fields to tight relative tolerances.  No GPU needed.
"""
import os

import numpy as np
import pytest

import oracle
from helpers import potential_up_to_constant, rel_err

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DAMP_NAMES = {0: "", 1: "AMOEBA", 2: "THOLE", 3: "ERF"}


@pytest.fixture(scope="module")
def tens():
    return np.load(os.path.join(GOLD, "ref_tensors.npz"))


@pytest.fixture(scope="module")
def fields():
    return np.load(os.path.join(GOLD, "ref_fields.npz"))


def _scale(pts, nmax):
    """Natural size of order-k tensor entries: (2k-1)!! / r^(k+1)."""
    r = np.linalg.norm(pts[:, :3], axis=1)
    cols = []
    for k in range(nmax + 1):
        s = np.prod(np.arange(1, 2 * k, 2)) / r ** (k + 1) if k else 1 / r
        cols += [s] * ((k + 1) * (k + 2) // 2)
    return np.array(cols).T


def test_cnij_int32_table_bit_exact(tens):
    """set_Cnij_coefficients with integer(ip) = int32 (tensors_recursive.F90:64-93)."""
    ref = tens["cnij32"]
    mine = oracle.cnij(16, wrap32=True)
    assert ref.shape == mine.shape
    assert np.array_equal(ref.astype(np.float64), mine)
    # the default build's table really wraps (orders >= 11)
    assert not np.array_equal(tens["cnij32"], tens["cnij64"])


def test_cnij_int64_table_matches_exact_mode(tens):
    """A -DINT64 build's table equals the oracle's exact coefficients wherever
    those fit in 53 bits (the table's top rows, i = 17, which order-16
    tensors never read, overflow even int64)."""
    ex = oracle.cnij(16, wrap32=False)
    ok = np.abs(ex) < 2.0 ** 53
    assert ok.mean() > 0.9
    assert np.array_equal(tens["cnij64"][ok].astype(np.float64), ex[ok])


def test_tn_recursive_ref_mode(tens):
    """Tn_recursive at order 16 with the wrapped table (what gfortran builds
    evaluate for every undamped tensor) against the oracle's ref mode."""
    pts = tens["none_pts"]
    ref = tens["none_rec32"]
    T = oracle.tensors(16, pts[:, 0], pts[:, 1], pts[:, 2], "", coef="ref")
    scale = np.maximum(_scale(pts, 16), np.abs(ref))
    assert np.max(np.abs(T - ref) / scale) < 1e-13


def test_tn_recursive_int64_matches_exact_mode(tens):
    pts = tens["none_pts"]
    ref = tens["none_rec64"]
    T = oracle.tensors(16, pts[:, 0], pts[:, 1], pts[:, 2], "", coef="exact")
    assert np.max(np.abs(T - ref) / _scale(pts, 16)) < 1e-12


def test_generated_undamped_tensors_exact_mode(tens):
    """The generated closed forms T0..T12 of tensors.F90 (50-digit values)."""
    pts = tens["none_pts"]
    ref = tens["none_gen"]
    T = oracle.tensors(12, pts[:, 0], pts[:, 1], pts[:, 2], "", coef="exact")
    assert np.max(np.abs(T - ref) / _scale(pts, 12)) < 1e-13


@pytest.mark.parametrize("kind", ["AMOEBA", "THOLE", "ERF"])
@pytest.mark.parametrize("coef", ["ref", "exact"])
def test_generated_damped_tensors(tens, kind, coef):
    """Tn_damp_{amoeba,thole,erf} order 6 (50-digit values of the reference's
    formulas) against the oracle's radial recursion, both coefficient modes."""
    pts = tens[kind + "_pts"]
    ref = tens[kind + "_gen"]
    T = oracle.tensors(6, pts[:, 0], pts[:, 1], pts[:, 2], kind, pts[:, 3], coef=coef)
    assert np.max(np.abs(T - ref) / _scale(pts, 6)) < 1e-13


@pytest.mark.parametrize("kind", ["AMOEBA", "THOLE", "ERF"])
def test_damped_tensors_within_reference_rounding(tens, kind):
    """What the reference computes in binary64 differs from its exact value
    only by its own rounding; the oracle lies within that band."""
    pts = tens[kind + "_pts"]
    ex, f64 = tens[kind + "_gen"], tens[kind + "_f64"]
    T = oracle.tensors(6, pts[:, 0], pts[:, 1], pts[:, 2], kind, pts[:, 3], coef="ref")
    sc = _scale(pts, 6)
    own = np.abs(f64 - ex) / sc
    assert np.all(np.abs(T - f64) / sc <= own + 1e-13)


def _case(fields, name):
    g = lambda k: fields[name + "_" + k]
    theta, ncrit, p, f, dcode = g("cfg")
    damp = DAMP_NAMES[int(dcode)]
    box = g("box")
    return dict(X=g("X"), M=g("M"), E=g("E"), d=g("d") if damp else None, theta=float(theta), ncrit=int(ncrit),
                p=int(p), f=int(f), damp=damp, periodic=bool(np.any(box)), box=box)


CASES = ["water_none", "water_thole", "water_amoeba", "uniform_erf", "uniform_charges", "uniform_octupole_f3",
         "water_octupole_thole_f3", "water_amoeba_f3", "uniform_octupole_erf"]
PERIODIC = ["periodic_cubic", "periodic_triclinic_thole", "periodic_amoeba_p6"]


@pytest.mark.parametrize("name", CASES)
def test_field_direct_matches_reference(fields, name):
    c = _case(fields, name)
    O = oracle.field_direct(0, c["X"], c["M"], c["E"], c["f"], c["damp"], c["d"])
    ref = fields[name + "_direct"]
    cols = slice(1, None) if c["damp"] == "AMOEBA" else slice(None)
    assert rel_err(O, ref, cols) <= 1e-12


@pytest.mark.parametrize("name", CASES + PERIODIC)
def test_field_fmm_matches_reference(fields, name):
    """field_fmm, including periodic cells (27 images, lattice sum, surface
    term; src/fmm.F90:884-979)."""
    c = _case(fields, name)
    O = oracle.field_fmm(0, c["X"], c["M"], c["E"], c["theta"], c["ncrit"], c["p"], c["f"], c["damp"], c["d"],
                         c["periodic"], c["box"])
    ref = fields[name + "_fmm"]
    assert np.all(np.isfinite(ref))
    assert rel_err(O, ref, slice(1, None)) <= 1e-12
    if c["periodic"]:
        # the potential up to a constant; in full where the lattice sum
        # converged (its constant is otherwise dominated by rounding)
        var, const = potential_up_to_constant(O, ref)
        assert var <= 1e-12
        if oracle.last_lattice_levels() < 50:
            assert rel_err(O, ref, slice(0, 1)) <= 1e-12
    elif c["damp"] != "AMOEBA":
        assert rel_err(O, ref, slice(0, 1)) <= 1e-12


@pytest.mark.parametrize("name", ["water_none", "water_thole"])
def test_tree_and_lists_match_reference(fields, name):
    c = _case(fields, name)
    t = oracle.tree(c["X"], c["ncrit"], c["theta"], centroid="sequential")
    g = lambda k: fields[name + "_tree_" + k]
    assert np.array_equal(t["center"], g("center"))
    assert np.array_equal(t["r"], g("r"))
    assert np.array_equal(t["rmax"], g("rmax"))
    for k, kk in (("depth", "depth"), ("parent", "parent"), ("is_leaf", "leaf"), ("count", "count")):
        assert np.array_equal(t[k], g(kk)), k
    assert np.array_equal(t["far"], g("far"))
    assert np.array_equal(t["near"], g("near"))


# ---------------------------------------------------------------- QM/MM helpers

def test_qmmm_helpers_stop_in_the_reference(fields):
    """As shipped, the reference's helpers stop in their final clean-up
    (finalize deallocates interaction lists they never build); the fixture's
    outputs were read with that DEALLOCATE skipped."""
    stops = [str(x) for x in fields["qmmm_stops"]]
    assert len(stops) == 3 and all("DEALLOCATE" in x for x in stops)


def test_qmmm_get_boxes_matches_reference(fields):
    th, nc, p, f = fields["qmmm_cfg"]
    idx, bc, bi = oracle.get_boxes(fields["qmmm_X"], fields["qmmm_T"], th, int(nc), int(p))
    assert np.array_equal(idx, fields["qmmm_idx_near"])
    assert np.array_equal(bc, fields["qmmm_box_coordinates"])
    assert np.array_equal(bi, fields["qmmm_box_indices"])


def test_qmmm_get_multipoles_matches_reference(fields):
    th, nc, p, f = fields["qmmm_cfg"]
    idx, bc, bm = oracle.get_multipoles(0, fields["qmmm_X"], fields["qmmm_M"], fields["qmmm_T"], th, int(nc), int(p))
    assert np.array_equal(idx, fields["qmmm_idx_near_mp"])
    assert np.array_equal(bc, fields["qmmm_box_coordinates_mp"])
    ref = fields["qmmm_box_multipoles"]
    assert np.max(np.abs(bm - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_qmmm_interpolate_electron_fields_matches_reference(fields):
    th, nc, p, f = fields["qmmm_cfg"]
    F = oracle.interpolate_electron_fields(0, fields["qmmm_X"], fields["qmmm_local"], fields["qmmm_box_indices"], th,
                                           int(nc), int(p), int(f))
    ref = fields["qmmm_field"]
    assert np.linalg.norm(F - ref) <= 1e-12 * np.linalg.norm(ref)

"""The C ABI library loads and exports every symbol include/fmm_gpu.h
declares; host-side argument checks reject bad input before any device work.
None of these tests needs a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "fmm_gpu.h")).read()
    return sorted(set(re.findall(r"\b(fmm_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def L():
    from fmm_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from fmm_gb300 import build
        build.build()
    return _lib.lib()


def test_every_declared_symbol_is_exported(L):
    names = _declared()
    assert len(names) >= 9
    for n in names:
        assert hasattr(L, n), n


def test_python_binding_covers_header():
    from fmm_gb300 import _lib
    for n in _lib.EXPORTED:
        assert n in _declared()


def test_strerror_and_version(L):
    from fmm_gb300 import _lib
    assert "invalid" in _lib.strerror(_lib.FMM_EINVAL)
    assert b"sm_103a" in L.fmm_version()


def _call_fmm(L, n=10, damp=b"", exw=1, excl=None, periodic=0, mdim=10, f=1):
    X = np.zeros((n, 3), order="F")
    M = np.zeros((n, mdim), order="F")
    E = excl if excl is not None else np.zeros((n, exw), dtype=np.int32, order="F")
    F = np.zeros((n, 4), order="F")
    d = ctypes.POINTER(ctypes.c_double)
    return L.fmm_field_fmm(0, n, X.ctypes.data_as(d), mdim, M.ctypes.data_as(d), E.shape[1],
                           E.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 0.5, 4, 5, f, F.ctypes.data_as(d), damp,
                           len(damp), None, periodic, None, None)


def test_host_side_argument_checks(L):
    from fmm_gb300 import _lib
    assert _call_fmm(L, damp=b"NOPE") == _lib.FMM_EINVAL
    assert _call_fmm(L, damp=b"THOLE") == _lib.FMM_EINVAL  # damping factors missing
    bad = np.full((10, 1), 11, dtype=np.int32, order="F")
    assert _call_fmm(L, excl=bad) == _lib.FMM_EINVAL
    assert _call_fmm(L, excl=-bad) == _lib.FMM_EINVAL
    assert _call_fmm(L, mdim=7) == _lib.FMM_EINVAL
    assert _call_fmm(L, mdim=35) == _lib.FMM_ENOTSUP  # multipole order 4
    assert _call_fmm(L, f=4) == _lib.FMM_ENOTSUP
    assert _call_fmm(L, periodic=1) == _lib.FMM_EINVAL  # periodic without a box matrix


def test_product_path_has_no_oracle_dependency():
    for d, _, files in os.walk(os.path.join(ROOT, "fmm_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                txt = open(os.path.join(d, f)).read()
                assert "import oracle" not in txt and "from oracle" not in txt, f
                assert "liboracle" not in txt, f


def test_stats_vector_matches_the_python_names(L):
    """fmm_last_stats (host-side, no GPU needed) writes exactly the entries
    the Python binding names, in the documented count."""
    import fmm_gb300
    buf = (ctypes.c_double * 64)()
    k = L.fmm_last_stats(buf, 64)
    assert k == len(fmm_gb300.STAT_NAMES) == 42
    assert fmm_gb300.STAT_NAMES[-2:] == ["corr_leaf_pairs", "corr_particle_pairs"]
    txt = open(os.path.join(ROOT, "include", "fmm_gpu.h")).read()
    assert "at most 42" in txt

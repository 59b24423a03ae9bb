"""ctypes front end of the CPU oracle (test infrastructure only).

The call signatures mirror the reference's f2py interface
(``octree.fmm.field_fmm`` / ``field_direct``, src/fmm.F90:1338-1400), plus
keyword options that select reference or exact behaviour (see the header of
fmm_oracle.cpp).
"""
import ctypes
import os

import numpy as np

from . import build as _build

__all__ = ["field_direct", "field_fmm", "tensors", "radial_g", "tree", "cnij", "DAMP", "n_components"]

DAMP = {"": 0, "AMOEBA": 1, "THOLE": 2, "ERF": 3}


class _Opts(ctypes.Structure):
    _fields_ = [("coef_mode", ctypes.c_int), ("excl_mode", ctypes.c_int),
                ("centroid_mode", ctypes.c_int), ("nthreads", ctypes.c_int), ("mac_mode", ctypes.c_int),
                ("target_rel_err", ctypes.c_double)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        d = ctypes.POINTER(ctypes.c_double)
        i32 = ctypes.POINTER(ctypes.c_int32)
        i64 = ctypes.c_int64
        lib.oracle_field_direct.argtypes = [i64, d, ctypes.c_int, d, ctypes.c_int, i32, ctypes.c_int, d,
                                            ctypes.c_int, d, ctypes.POINTER(_Opts)]
        lib.oracle_field_fmm.argtypes = [i64, d, ctypes.c_int, d, ctypes.c_int, i32, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, d, ctypes.c_int, d, ctypes.c_int,
                                         ctypes.POINTER(_Opts)]
        lib.oracle_tensors.argtypes = [ctypes.c_int, i64, d, d, d, ctypes.c_int, d, ctypes.c_int, d]
        lib.oracle_radial_g.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, d]
        lib.oracle_tree_build.restype = ctypes.c_void_p
        lib.oracle_tree_build.argtypes = [i64, d, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_int)]
        lib.oracle_tree_sizes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
        lib.oracle_tree_get.argtypes = [ctypes.c_void_p, d, d, d, i32, i32, i32, i32, i32, i32, i32]
        lib.oracle_tree_free.argtypes = [ctypes.c_void_p]
        lib.oracle_cnij.argtypes = [ctypes.c_int, ctypes.c_int, d]
        _lib = lib
    return _lib


def n_components(order):
    return (order + 1) * (order + 2) * (order + 3) // 6


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _opts(coef_mode="ref", excl_mode="ref", centroid_mode="sequential", nthreads=0, mac_mode="ref",
          target_rel_err=1e-6):
    return _Opts({"ref": 0, "exact": 1}[coef_mode], {"ref": 0, "mask": 1}[excl_mode],
                 {"sequential": 0, "blocked": 1}[centroid_mode], int(nthreads), {"ref": 0, "damping": 1}[mac_mode],
                 float(target_rel_err))


def _prep(coordinates, multipoles, exclusions, damp_type, damping_factors):
    X = np.asfortranarray(coordinates, dtype=np.float64)
    M = np.asfortranarray(multipoles, dtype=np.float64)
    E = np.asfortranarray(exclusions, dtype=np.int32)
    if E.ndim == 1:
        E = E.reshape(-1, 1, order="F")
    dt = damp_type.strip().upper() if damp_type else ""
    if dt not in DAMP:
        raise RuntimeError("Unknown damp type: " + damp_type)
    d = np.ascontiguousarray(damping_factors if damping_factors is not None else np.zeros(X.shape[0]),
                             dtype=np.float64)
    if d.size < X.shape[0]:
        d = np.zeros(X.shape[0])
    return X, M, E, DAMP[dt], d


def field_direct(comm, coordinates, multipoles, exclusions, field_order, damp_type="", damping_factors=None, **kw):
    X, M, E, dt, d = _prep(coordinates, multipoles, exclusions, damp_type, damping_factors)
    n = X.shape[0]
    F = np.zeros((n, n_components(field_order)), order="F")
    o = _opts(**kw)
    st = _load().oracle_field_direct(n, _dp(X), M.shape[1], _dp(M), E.shape[1], _ip(E), int(field_order), _dp(F),
                                     dt, _dp(d), ctypes.byref(o))
    if st != 0:
        raise RuntimeError("oracle field_direct failed with status %d" % st)
    return F


def field_fmm(comm, coordinates, multipoles, exclusions, theta, ncrit, expansion_order, field_order, damp_type="",
              damping_factors=None, is_periodic=False, box_matrix=None, **kw):
    X, M, E, dt, d = _prep(coordinates, multipoles, exclusions, damp_type, damping_factors)
    n = X.shape[0]
    F = np.zeros((n, n_components(field_order)), order="F")
    o = _opts(**kw)
    st = _load().oracle_field_fmm(n, _dp(X), M.shape[1], _dp(M), E.shape[1], _ip(E), float(theta), int(ncrit),
                                  int(expansion_order), int(field_order), _dp(F), dt, _dp(d), int(bool(is_periodic)),
                                  ctypes.byref(o))
    if st != 0:
        raise RuntimeError("oracle field_fmm failed with status %d" % st)
    return F


def tensors(nmax, x, y, z, damp_type="", a=None, coef="ref"):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    z = np.ascontiguousarray(z, dtype=np.float64)
    a = np.ascontiguousarray(a if a is not None else np.zeros_like(x), dtype=np.float64)
    T = np.zeros((x.size, n_components(nmax)), order="F")
    st = _load().oracle_tensors(int(nmax), x.size, _dp(x), _dp(y), _dp(z), DAMP[damp_type], _dp(a),
                                {"ref": 0, "exact": 1}[coef], _dp(T))
    if st != 0:
        raise RuntimeError("oracle tensors failed")
    return T


def radial_g(damp_type, r, a, n):
    g = np.zeros(n + 1)
    _load().oracle_radial_g(DAMP[damp_type], float(r), float(a), int(n), _dp(g))
    return g


def tree(coordinates, ncrit, theta, centroid="sequential"):
    """Reference octree and interaction lists (DFS node ids) as numpy arrays."""
    X = np.asfortranarray(coordinates, dtype=np.float64)
    n = X.shape[0]
    lib = _load()
    st = ctypes.c_int(0)
    h = lib.oracle_tree_build(n, _dp(X), int(ncrit), float(theta), {"sequential": 0, "blocked": 1}[centroid],
                              ctypes.byref(st))
    if not h:
        raise RuntimeError("oracle tree build failed with status %d" % st.value)
    try:
        sz = np.zeros(4, dtype=np.int64)
        lib.oracle_tree_sizes(h, sz.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        M, nf, nn, md = (int(v) for v in sz)
        out = dict(center=np.zeros((M, 3)), r=np.zeros(M), rmax=np.zeros(M), depth=np.zeros(M, np.int32),
                   parent=np.zeros(M, np.int32), is_leaf=np.zeros(M, np.int32), count=np.zeros(M, np.int32),
                   leaf_of=np.zeros(n, np.int32), far=np.zeros((nf, 2), np.int32),
                   near=np.zeros((nn, 2), np.int32))
        lib.oracle_tree_get(h, _dp(out["center"]), _dp(out["r"]), _dp(out["rmax"]), _ip(out["depth"]),
                            _ip(out["parent"]), _ip(out["is_leaf"]), _ip(out["count"]), _ip(out["leaf_of"]),
                            _ip(out["far"]), _ip(out["near"]))
        out["max_depth"] = md
        return out
    finally:
        lib.oracle_tree_free(h)


def cnij(maxo, wrap32=True):
    """The Cnij table Cnij(1:2*maxo+3, 0:maxo+1, 0:maxo+1) of
    tensors_recursive.F90:64-93, as a Fortran-ordered float64 array."""
    out = np.zeros((2 * maxo + 3, maxo + 2, maxo + 2), order="F")
    _load().oracle_cnij(int(maxo), int(bool(wrap32)), _dp(out))
    return out

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

__all__ = ["field_direct", "field_fmm", "tensors", "radial_g", "tree", "cnij", "get_boxes", "get_multipoles",
           "interpolate_electron_fields", "last_lattice_levels", "DAMP", "n_components"]

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
        lib.oracle_field_fmm_box.argtypes = [i64, d, ctypes.c_int, d, ctypes.c_int, i32, ctypes.c_double,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int, d, ctypes.c_int, d,
                                             ctypes.c_int, d, ctypes.POINTER(_Opts)]
        lib.oracle_tensors.argtypes = [ctypes.c_int, i64, d, d, d, ctypes.c_int, d, ctypes.c_int, d]
        lib.oracle_radial_g.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, d]
        lib.oracle_tree_build.restype = ctypes.c_void_p
        lib.oracle_tree_build.argtypes = [i64, d, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_int)]
        lib.oracle_tree_sizes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
        lib.oracle_tree_get.argtypes = [ctypes.c_void_p, d, d, d, i32, i32, i32, i32, i32, i32, i32]
        lib.oracle_tree_free.argtypes = [ctypes.c_void_p]
        lib.oracle_cnij.argtypes = [ctypes.c_int, ctypes.c_int, d]
        lib.oracle_last_lattice_levels.restype = ctypes.c_int
        i64p = ctypes.POINTER(ctypes.c_int64)
        lib.oracle_get_boxes.argtypes = [i64, d, i64, d, ctypes.c_double, ctypes.c_int, i64p, i32, d, i32]
        lib.oracle_get_multipoles.argtypes = [i64, d, ctypes.c_int, ctypes.c_int, d, i64, d, ctypes.c_double,
                                              ctypes.c_int, ctypes.c_int, i64p, i32, d, d]
        lib.oracle_interpolate_electron_fields.argtypes = [i64, d, i64, ctypes.c_int, d, i32, ctypes.c_double,
                                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, d]
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
    box = None
    if is_periodic:
        box = np.asfortranarray(box_matrix, dtype=np.float64)
    st = _load().oracle_field_fmm_box(n, _dp(X), M.shape[1], _dp(M), E.shape[1], _ip(E), float(theta), int(ncrit),
                                      int(expansion_order), int(field_order), _dp(F), dt, _dp(d),
                                      int(bool(is_periodic)), _dp(box) if box is not None else None,
                                      ctypes.byref(o))
    if st != 0:
        raise RuntimeError("oracle field_fmm failed with status %d" % st)
    return F


def last_lattice_levels():
    """Lattice levels the last periodic field_fmm used (50 = the reference's
    limit, reached when its convergence test never passes)."""
    return int(_load().oracle_last_lattice_levels())


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


def _i64p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def get_boxes(coordinates, target_coordinates, theta, ncrit, expansion_order):
    """get_boxes (src/fmm.F90:1258-1308): (idx_near_field, box_coordinates,
    box_indices), 1-based indices as in the reference."""
    X = np.asfortranarray(coordinates, dtype=np.float64)
    T = np.asfortranarray(target_coordinates, dtype=np.float64)
    sz = np.zeros(2, dtype=np.int64)
    lib = _load()
    st = lib.oracle_get_boxes(X.shape[0], _dp(X), T.shape[0], _dp(T), float(theta), int(ncrit), _i64p(sz), None, None,
                              None)
    if st != 0:
        raise RuntimeError("oracle get_boxes failed with status %d" % st)
    idx = np.zeros(max(1, sz[0]), dtype=np.int32)
    bc = np.zeros((max(1, sz[1]), 3), order="F") if not sz[1] else np.zeros((int(sz[1]), 3), order="F")
    bi = np.zeros(max(1, sz[1]), dtype=np.int32)
    lib.oracle_get_boxes(X.shape[0], _dp(X), T.shape[0], _dp(T), float(theta), int(ncrit), _i64p(sz), _ip(idx),
                         _dp(bc), _ip(bi))
    return idx[:sz[0]], bc[:sz[1]], bi[:sz[1]]


def get_multipoles(comm, coordinates, multipoles, target_coordinates, theta, ncrit, expansion_order):
    """get_multipoles (src/fmm.F90:1173-1256): (idx_near_field,
    box_coordinates, box_multipoles); multipoles (N, dim, ndens)."""
    X = np.asfortranarray(coordinates, dtype=np.float64)
    Mp = np.asfortranarray(multipoles, dtype=np.float64)
    if Mp.ndim == 2:
        Mp = Mp.reshape(Mp.shape + (1,), order="F")
    T = np.asfortranarray(target_coordinates, dtype=np.float64)
    n, dim, nd = Mp.shape
    sz = np.zeros(2, dtype=np.int64)
    lib = _load()
    args = (n, _dp(X), dim, nd, _dp(Mp), T.shape[0], _dp(T), float(theta), int(ncrit), int(expansion_order))
    st = lib.oracle_get_multipoles(*args, _i64p(sz), None, None, None)
    if st != 0:
        raise RuntimeError("oracle get_multipoles failed with status %d" % st)
    idx = np.zeros(max(1, sz[0]), dtype=np.int32)
    nb = max(1, int(sz[1]))
    bc = np.zeros((nb, 3), order="F")
    bm = np.zeros((nb, n_components(expansion_order), nd), order="F")
    if sz[1]:
        bc = np.zeros((int(sz[1]), 3), order="F")
        bm = np.zeros((int(sz[1]), n_components(expansion_order), nd), order="F")
    lib.oracle_get_multipoles(*args, _i64p(sz), _ip(idx), _dp(bc), _dp(bm))
    return idx[:sz[0]], bc[:sz[1]], bm[:sz[1]]


def interpolate_electron_fields(comm, coordinates, local_expansion, box_indices, theta, ncrit, expansion_order,
                                field_order):
    """interpolate_electron_fields (src/fmm.F90:1310-1336): the field
    (N, nT(field_order), ndens) of local expansions given at boxes."""
    X = np.asfortranarray(coordinates, dtype=np.float64)
    Lx = np.asfortranarray(local_expansion, dtype=np.float64)
    if Lx.ndim == 2:
        Lx = Lx.reshape(Lx.shape + (1,), order="F")
    bi = np.ascontiguousarray(box_indices, dtype=np.int32)
    n = X.shape[0]
    F = np.zeros((n, n_components(field_order), Lx.shape[2]), order="F")
    st = _load().oracle_interpolate_electron_fields(n, _dp(X), Lx.shape[0], Lx.shape[2], _dp(Lx), _ip(bi),
                                                     float(theta), int(ncrit), int(expansion_order),
                                                     int(field_order), _dp(F))
    if st != 0:
        raise RuntimeError("oracle interpolate_electron_fields failed with status %d" % st)
    return F

"""GB300-native (sm_103a) field evaluation for Cartesian-multipole FMM.

Drop-in for the field-evaluation path of peter-reinholdt/fmm
(``field_direct`` / ``field_fmm``, src/fmm.F90:1338-1400).  The functions
here take the reference's arguments in the reference's order and layouts;
extra behaviour is selected through keyword-only ``Options``.

All arithmetic runs in the CUDA library ``libfmm_gb300.so`` (built in-tree by
``fmm_gb300.build``); there is no CPU code path.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import FmmError

__all__ = ["field_direct", "field_fmm", "field_fmm_batched", "field_direct_device", "field_fmm_device", "Options",
           "last_stats", "n_components", "FmmError", "version", "load_selector", "release_workspace", "get_boxes",
           "get_multipoles", "interpolate_electron_fields", "Plan",
           "set_p2p_shape"]


def n_components(order):
    """Packed components of all orders <= order: (k+1)(k+2)(k+3)/6."""
    return (order + 1) * (order + 2) * (order + 3) // 6


@dataclass
class Options:
    """Behaviour switches that the reference API does not have.

    The defaults reproduce the reference (int32 Cnij closed form in M2L,
    excluded sources at R = 1e10, reference MAC, FP64, fixed order)."""

    coef_mode: str = "ref"        # "ref" | "exact"
    excl_mode: str = "ref"        # "ref" (1e10 displacement) | "mask"
    precision: str = "fp64"       # "fp64" | "mixed" | "mixed_near" | "mixed_far"
    centroid_mode: str = "sequential"  # "sequential" | "blocked"
    mac_mode: str = "ref"         # "ref" | "damping"
    selector: str = "fixed"       # "fixed" | "learned"
    target_rel_err: float = 1e-6
    stream: int = 0               # cudaStream_t for the *_device calls
    autotune: bool = False        # ncrit and near-field launch shape timed per class of calls

    @classmethod
    def exact(cls, **kw):
        d = dict(coef_mode="exact", excl_mode="mask", centroid_mode="blocked")
        d.update(kw)
        return cls(**d)

    def to_c(self):
        o = _lib.FmmOpts()
        o.version = 1
        o.coef_mode = {"ref": 0, "exact": 1}[self.coef_mode]
        o.excl_mode = {"ref": 0, "mask": 1}[self.excl_mode]
        o.precision = {"fp64": 0, "mixed": 1, "mixed_near": 2, "mixed_far": 3}[self.precision]
        o.centroid_mode = {"sequential": 0, "blocked": 1}[self.centroid_mode]
        o.mac_mode = {"ref": 0, "damping": 1}[self.mac_mode]
        o.selector = {"fixed": 0, "learned": 1}[self.selector]
        o.target_rel_err = float(self.target_rel_err)
        o.stream = int(self.stream) or None
        o.autotune = 1 if self.autotune else 0
        return o


import os
import threading

SELECTOR_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "selector_v2.bin")
_sel_local = threading.local()


def load_selector(path=None):
    """Loads the expansion-order selector's network parameters (float32 blob
    written by fmm_gb300.selector_train) for the calling thread."""
    path = path or SELECTOR_WEIGHTS
    if not os.path.exists(path):
        raise FmmError(_lib.FMM_ENOTSUP, "learned selector (no weights at %s; run fmm_gb300.selector_train)" % path)
    p = np.fromfile(path, dtype="<f4")
    L = _lib.lib()
    L.fmm_selector_load.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    _lib.check(L.fmm_selector_load(p.ctypes.data, p.size), "fmm_selector_load")
    _sel_local.loaded = path


def _options_c(options):
    opts = options or Options()
    if opts.selector == "learned" and getattr(_sel_local, "loaded", None) is None:
        load_selector()
    return opts.to_c()


def _damp_bytes(damp_type):
    s = (damp_type or "").encode()
    return s, len(s)


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _prep(coordinates, multipoles, exclusions, damping_factors):
    X = np.asfortranarray(coordinates, dtype=np.float64)
    if X.ndim != 2 or X.shape[1] != 3:
        raise ValueError("coordinates must be (N, 3)")
    n = X.shape[0]
    M = np.asfortranarray(multipoles, dtype=np.float64)
    if M.ndim == 1:
        M = M.reshape(n, 1, order="F")
    if M.shape[0] != n:
        raise ValueError("multipoles must be (N, dim)")
    E = np.asfortranarray(exclusions, dtype=np.int32)
    if E.ndim == 1:
        E = E.reshape(n, -1, order="F")
    if E.shape[0] != n:
        raise ValueError("exclusions must be (N, width)")
    d = None
    if damping_factors is not None and np.size(damping_factors) > 0:
        d = np.ascontiguousarray(damping_factors, dtype=np.float64)
        if d.size < n:
            raise ValueError("damping_factors must have N entries")
    return X, M, E, d


def field_direct(comm, coordinates, multipoles, exclusions, field_order, damp_type="", damping_factors=None, *,
                 options=None):
    """Direct-sum field, ``fmm::field_direct`` (src/fmm.F90:1338-1352).

    Returns the (N, nT(field_order)) Fortran-ordered field array."""
    X, M, E, d = _prep(coordinates, multipoles, exclusions, damping_factors)
    n = X.shape[0]
    F = np.zeros((n, n_components(field_order)), order="F")
    ds, dl = _damp_bytes(damp_type)
    o = (options or Options()).to_c()
    st = _lib.lib().fmm_field_direct(int(comm or 0), n, _dptr(X), M.shape[1], _dptr(M), E.shape[1],
                                     E.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), int(field_order), _dptr(F),
                                     ds, dl, _dptr(d) if d is not None else None, ctypes.byref(o))
    _lib.check(st, "field_direct")
    return F


def field_fmm(comm, coordinates, multipoles, exclusions, theta, ncrit, expansion_order, field_order, damp_type="",
              damping_factors=None, is_periodic=False, box_matrix=None, *, options=None):
    """FMM field, ``fmm::field_fmm`` (src/fmm.F90:1354-1400).

    Returns the (N, nT(field_order)) Fortran-ordered field array."""
    X, M, E, d = _prep(coordinates, multipoles, exclusions, damping_factors)
    n = X.shape[0]
    F = np.zeros((n, n_components(field_order)), order="F")
    ds, dl = _damp_bytes(damp_type)
    o = _options_c(options)
    box = None
    if box_matrix is not None:
        box = np.asfortranarray(box_matrix, dtype=np.float64)
    st = _lib.lib().fmm_field_fmm(int(comm or 0), n, _dptr(X), M.shape[1], _dptr(M), E.shape[1],
                                  E.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), float(theta), int(ncrit),
                                  int(expansion_order), int(field_order), _dptr(F), ds, dl,
                                  _dptr(d) if d is not None else None, int(bool(is_periodic)),
                                  _dptr(box) if box is not None else None, ctypes.byref(o))
    _lib.check(st, "field_fmm")
    return F


def set_p2p_shape(threads=0, stage=0, queue=0):
    """Launch shape of the mixed-precision near field for this thread's later
    calls (fmm_set_p2p_shape); no arguments restores the default."""
    _lib.check(_lib.lib().fmm_set_p2p_shape(int(threads), int(stage), int(queue)), "set_p2p_shape")


class Plan:
    """Fixed coordinates, many multipole sets (fmm_plan_create / execute).

    The octree, interaction lists and M2L grouping are built once; every
    ``execute(multipoles)`` replays one captured CUDA graph and returns the
    field ``field_fmm`` gives for the same inputs.  Arguments as
    ``field_fmm`` without the multipoles (``dim`` = their column count);
    fixed acceptance rule only.  ``close()`` (or garbage collection) frees
    the plan's device memory."""

    def __init__(self, coordinates, dim, exclusions, theta, ncrit, expansion_order, field_order, damp_type="",
                 damping_factors=None, *, options=None):
        X, _, E, d = _prep(coordinates, np.zeros(np.shape(coordinates)[0]), exclusions, damping_factors)
        n = X.shape[0]
        ds, dl = _damp_bytes(damp_type)
        o = _options_c(options)
        h = ctypes.c_void_p(None)
        L = _lib.lib()
        st = L.fmm_plan_create(n, _dptr(X), int(dim), E.shape[1], E.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                               float(theta), int(ncrit), int(expansion_order), int(field_order), ds, dl,
                               _dptr(d) if d is not None else None, ctypes.byref(o), ctypes.byref(h))
        _lib.check(st, "plan_create")
        self._h = h
        self._lib = L
        self.n, self.dim, self.field_order = n, int(dim), int(field_order)

    @classmethod
    def batched(cls, systems_list, dim, theta, ncrit, expansion_order, field_order, damp_type="", *, options=None):
        """A plan over independent systems packed as ``field_fmm_batched``
        packs them (dicts with coordinates, exclusions, damping_factors);
        ``execute_systems`` takes and returns per-system arrays."""
        sizes = [np.asarray(s["coordinates"]).shape[0] for s in systems_list]
        offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        n = int(offsets[-1])
        X = np.asfortranarray(np.concatenate([np.asarray(s["coordinates"], dtype=np.float64) for s in systems_list]))
        width = max(np.asarray(s["exclusions"]).reshape(sizes[k], -1).shape[1] for k, s in enumerate(systems_list))
        E = np.zeros((n, width), dtype=np.int32, order="F")
        for k, s in enumerate(systems_list):
            e = np.asarray(s["exclusions"], dtype=np.int32).reshape(sizes[k], -1)
            E[offsets[k]:offsets[k + 1], :e.shape[1]] = e
        d = None
        if damp_type:
            d = np.ascontiguousarray(np.concatenate([np.asarray(s["damping_factors"], dtype=np.float64)
                                                     for s in systems_list]))
        ds, dl = _damp_bytes(damp_type)
        o = _options_c(options)
        h = ctypes.c_void_p(None)
        L = _lib.lib()
        st = L.fmm_plan_create_batched(len(systems_list), offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                       _dptr(X), int(dim), E.shape[1], E.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                       float(theta), int(ncrit), int(expansion_order), int(field_order), ds, dl,
                                       _dptr(d) if d is not None else None, ctypes.byref(o), ctypes.byref(h))
        _lib.check(st, "plan_create_batched")
        obj = cls.__new__(cls)
        obj._h, obj._lib = h, L
        obj.n, obj.dim, obj.field_order = n, int(dim), int(field_order)
        obj.offsets = offsets
        return obj

    def execute_systems(self, multipoles_list):
        """Per-system multipoles in, per-system fields out (batched plans)."""
        M = np.asfortranarray(np.concatenate([np.asarray(m, dtype=np.float64).reshape(-1, self.dim)
                                              for m in multipoles_list]))
        F = self.execute(M)
        o = self.offsets
        return [F[o[k]:o[k + 1]] for k in range(len(o) - 1)]

    @property
    def kernels(self):
        """Kernel launches per evaluation (nodes of the captured graph)."""
        return self._lib.fmm_plan_kernels(self._h)

    def execute(self, multipoles, out=None):
        M = np.asfortranarray(multipoles, dtype=np.float64)
        if M.shape != (self.n, self.dim):
            raise ValueError("multipoles must have shape (%d, %d)" % (self.n, self.dim))
        F = out if out is not None else np.zeros((self.n, n_components(self.field_order)), order="F")
        st = self._lib.fmm_plan_execute(self._h, _dptr(M), _dptr(F))
        _lib.check(st, "plan_execute")
        return F

    def execute_device(self, multipoles, field):
        """Device arrays (anything with ``data_ptr()``), column-major."""
        st = self._lib.fmm_plan_execute_device(self._h, ctypes.c_void_p(int(multipoles.data_ptr())),
                                               ctypes.c_void_p(int(field.data_ptr())))
        _lib.check(st, "plan_execute_device")
        return field

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fmm_plan_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def field_fmm_batched(systems_list, theta, ncrit, expansion_order, field_order, damp_type="", *, options=None):
    """Many independent systems in one call (fmm_field_fmm_batched).

    `systems_list` is a sequence of dicts with the keys of fmm_gb300.systems
    (coordinates, multipoles, exclusions, damping_factors); exclusion indices
    are 1-based within each system.  Returns a list of per-system field
    arrays."""
    sizes = [np.asarray(s["coordinates"]).shape[0] for s in systems_list]
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    n = int(offsets[-1])
    X = np.asfortranarray(np.concatenate([np.asarray(s["coordinates"], dtype=np.float64) for s in systems_list]))
    M = np.asfortranarray(np.concatenate([np.asarray(s["multipoles"], dtype=np.float64) for s in systems_list]))
    width = max(np.asarray(s["exclusions"]).reshape(sizes[k], -1).shape[1] for k, s in enumerate(systems_list))
    E = np.zeros((n, width), dtype=np.int32, order="F")
    for k, s in enumerate(systems_list):
        e = np.asarray(s["exclusions"], dtype=np.int32).reshape(sizes[k], -1)
        E[offsets[k]:offsets[k + 1], :e.shape[1]] = e
    d = None
    if damp_type:
        d = np.ascontiguousarray(np.concatenate([np.asarray(s["damping_factors"], dtype=np.float64)
                                                 for s in systems_list]))
    F = np.zeros((n, n_components(field_order)), order="F")
    ds, dl = _damp_bytes(damp_type)
    o = _options_c(options)
    st = _lib.lib().fmm_field_fmm_batched(len(systems_list), offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                          _dptr(X), M.shape[1], _dptr(M), E.shape[1],
                                          E.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), float(theta), int(ncrit),
                                          int(expansion_order), int(field_order), _dptr(F), ds, dl,
                                          _dptr(d) if d is not None else None, ctypes.byref(o))
    _lib.check(st, "field_fmm_batched")
    return [F[offsets[k]:offsets[k + 1]] for k in range(len(systems_list))]


def _ptr(t):
    return None if t is None else ctypes.c_void_p(int(t.data_ptr()))


def field_direct_device(coordinates, multipoles, exclusions, field_order, field, damp_type="", damping_factors=None,
                        *, options=None):
    """Device-resident direct sum.  Arguments are CUDA tensors (anything with
    ``data_ptr()``) in the reference's column-major layouts; ``field`` is
    written.  Work is enqueued on ``options.stream``."""
    n = coordinates.shape[0]
    ds, dl = _damp_bytes(damp_type)
    o = (options or Options()).to_c()
    st = _lib.lib().fmm_field_direct_device(n, _ptr(coordinates), multipoles.shape[1], _ptr(multipoles),
                                            exclusions.shape[1], _ptr(exclusions), int(field_order), _ptr(field), ds,
                                            dl, _ptr(damping_factors), ctypes.byref(o))
    _lib.check(st, "field_direct_device")


def field_fmm_device(coordinates, multipoles, exclusions, theta, ncrit, expansion_order, field_order, field,
                     damp_type="", damping_factors=None, *, options=None):
    """Device-resident FMM (see ``field_direct_device``)."""
    n = coordinates.shape[0]
    ds, dl = _damp_bytes(damp_type)
    o = _options_c(options)
    st = _lib.lib().fmm_field_fmm_device(n, _ptr(coordinates), multipoles.shape[1], _ptr(multipoles),
                                         exclusions.shape[1], _ptr(exclusions), float(theta), int(ncrit),
                                         int(expansion_order), int(field_order), _ptr(field), ds, dl,
                                         _ptr(damping_factors), ctypes.byref(o))
    _lib.check(st, "field_fmm_device")


STAT_NAMES = ["num_nodes", "num_leaves", "max_depth", "m2l_pairs", "p2p_leaf_pairs", "p2p_particle_pairs", "t_tree",
              "t_p2m_m2m", "t_lists", "t_p2p", "t_m2l", "t_l2l_l2p", "t_total", "selector_fallback",
              "sampled_rms_err", "m2l_order_mean"] + ["m2l_pairs_q%d" % q for q in range(13)] + \
             ["t_p2p_kernel", "t_m2l_product", "m2l_groups", "list_candidates", "list_evals", "lattice_levels",
              "ncrit_used", "p2p_threads", "p2p_stage", "p2p_queue", "tuned", "corr_leaf_pairs", "corr_particle_pairs"]


def last_stats():
    """Sizes and per-phase device times (ms) of the last FMM call on this thread."""
    buf = (ctypes.c_double * len(STAT_NAMES))()
    k = _lib.lib().fmm_last_stats(buf, len(STAT_NAMES))
    return {STAT_NAMES[i]: buf[i] for i in range(k)}


def get_boxes(coordinates, target_coordinates, theta, ncrit, expansion_order, *, options=None):
    """``fmm::get_boxes`` (src/fmm.F90:1258-1308): returns (idx_near_field,
    box_coordinates, box_indices), indices 1-based as in the reference."""
    X = np.asfortranarray(coordinates, dtype=np.float64)
    T = np.asfortranarray(target_coordinates, dtype=np.float64)
    L = _lib.lib()
    sz = np.zeros(2, dtype=np.int64)
    o = (options or Options()).to_c()
    args = (X.shape[0], _dptr(X), T.shape[0], _dptr(T), float(theta), int(ncrit), int(expansion_order),
            sz.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    _lib.check(L.fmm_get_boxes(*args, None, None, None, ctypes.byref(o)), "get_boxes")
    idx = np.zeros(int(sz[0]), dtype=np.int32)
    bc = np.zeros((int(sz[1]), 3), order="F")
    bi = np.zeros(int(sz[1]), dtype=np.int32)
    _lib.check(L.fmm_get_boxes(*args, idx.ctypes.data, bc.ctypes.data, bi.ctypes.data, ctypes.byref(o)), "get_boxes")
    return idx, bc, bi


def get_multipoles(comm, coordinates, multipoles, target_coordinates, theta, ncrit, expansion_order, *, options=None):
    """``fmm::get_multipoles`` (src/fmm.F90:1173-1256): returns
    (idx_near_field, box_coordinates, box_multipoles); multipoles is
    (N, dim, ndens) (or (N, dim))."""
    X = np.asfortranarray(coordinates, dtype=np.float64)
    Mp = np.asfortranarray(multipoles, dtype=np.float64)
    if Mp.ndim == 2:
        Mp = Mp.reshape(Mp.shape + (1,), order="F")
    T = np.asfortranarray(target_coordinates, dtype=np.float64)
    n, dim, nd = Mp.shape
    L = _lib.lib()
    sz = np.zeros(2, dtype=np.int64)
    o = (options or Options()).to_c()
    args = (int(comm or 0), n, _dptr(X), dim, nd, _dptr(Mp), T.shape[0], _dptr(T), float(theta), int(ncrit),
            int(expansion_order), sz.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    _lib.check(L.fmm_get_multipoles(*args, None, None, None, ctypes.byref(o)), "get_multipoles")
    idx = np.zeros(int(sz[0]), dtype=np.int32)
    bc = np.zeros((int(sz[1]), 3), order="F")
    bm = np.zeros((int(sz[1]), n_components(expansion_order), nd), order="F")
    _lib.check(L.fmm_get_multipoles(*args, idx.ctypes.data, bc.ctypes.data, bm.ctypes.data, ctypes.byref(o)),
               "get_multipoles")
    return idx, bc, bm


def interpolate_electron_fields(comm, coordinates, local_expansion, box_indices, theta, ncrit, expansion_order,
                                field_order, *, options=None):
    """``fmm::interpolate_electron_fields`` (src/fmm.F90:1310-1336): the field
    (N, nT(field_order), ndens) of local expansions (nbox, nT(p), ndens) given
    at the 1-based nodes box_indices."""
    X = np.asfortranarray(coordinates, dtype=np.float64)
    Lx = np.asfortranarray(local_expansion, dtype=np.float64)
    if Lx.ndim == 2:
        Lx = Lx.reshape(Lx.shape + (1,), order="F")
    bi = np.ascontiguousarray(box_indices, dtype=np.int32)
    n = X.shape[0]
    F = np.zeros((n, n_components(field_order), Lx.shape[2]), order="F")
    o = (options or Options()).to_c()
    _lib.check(_lib.lib().fmm_interpolate_electron_fields(int(comm or 0), n, _dptr(X), Lx.shape[0], Lx.shape[2],
                                                          _dptr(Lx), bi.ctypes.data, float(theta), int(ncrit),
                                                          int(expansion_order), int(field_order), _dptr(F),
                                                          ctypes.byref(o)), "interpolate_electron_fields")
    return F


def release_workspace():
    """Frees the device memory the library holds for the calling thread
    (fmm_release_workspace); the next call allocates again."""
    _lib.check(_lib.lib().fmm_release_workspace(), "fmm_release_workspace")


def version():
    return _lib.lib().fmm_version().decode()

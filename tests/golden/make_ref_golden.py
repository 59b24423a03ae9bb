"""Golden fixtures produced by the reference's own source code.

The reference (peter-reinholdt/fmm) is Fortran; no Fortran compiler exists
on either machine of this project.  ``fortran_exec.py`` translates the
reference's source files statement by statement into Python and runs them,
so the numbers written here come from the reference's own statements:

ref_tensors.npz
  * ``cnij32`` / ``cnij64``: the Cnij table that ``set_Cnij_coefficients``
    (src/tensors_recursive.F90:64-93) builds for tensor order 16, with
    integer(ip) as int32 (the default build, where it wraps) and as int64;
  * ``none_pts`` with ``none_rec32`` / ``none_rec64`` (``Tn_recursive``,
    src/tensors_recursive.F90:95-135, order 16, the routine gfortran builds
    call for every undamped tensor, src/tensors.F90:12-16) and
    ``none_gen`` (the generated closed forms T0..T12 of src/tensors.F90,
    evaluated in 50-digit arithmetic: the exact value of the reference's
    formulas at the binary64 inputs);
  * per damping kind K in AMOEBA, THOLE, ERF: ``K_pts`` (x, y, z, a) with
    ``K_gen`` (Tn_damp_K order 6, src/tensors_damped_*.F90, 50 digits) and
    ``K_f64`` (the same statements in binary64, what the reference computes).
ref_fields.npz
  per case C: the inputs (``C_X``, ``C_M``, ``C_E``, ``C_d``), the settings
  (``C_cfg`` = [theta, ncrit, expansion_order, field_order, damp code]),
  ``C_direct`` (``field_direct``) and ``C_fmm`` (``field_fmm``) in binary64,
  and for the tree cases the reference's octree and interaction lists
  (``C_tree_*``: per DFS node centre, r, rmax, depth, parent, leaf flag,
  particle count; far and near lists as sorted (target, source) node pairs;
  node ids are the reference's DFS positions minus one); ``C_box`` is the
  periodic cell of the periodic cases (zero otherwise);
  ``qmmm_*``: get_boxes, get_multipoles (two multipole sets) and
  interpolate_electron_fields (two sets of local expansions) on one water
  system around six target points (src/fmm.F90:1134-1336), read with the
  DEALLOCATE that stops these helpers at their end skipped; ``qmmm_stops``
  records those stops.

Run where the reference source is present (the default path below, or
FMM_REFERENCE_SRC):  python tests/golden/make_ref_golden.py
Test infrastructure only; the tests read the .npz files, not the reference.
"""
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.environ.get("FMM_REFERENCE_SRC", "/root/reference/src")
FILES = ["tensors_recursive.F90", "tensors.F90", "tensors_damped_amoeba.F90", "tensors_damped_thole.F90",
         "tensors_damped_erf.F90", "fmm.F90"]
DAMP = {"": 0, "AMOEBA": 1, "THOLE": 2, "ERF": 3}

sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)


def _translated():
    import fortran_exec as fx
    return fx, fx.Translated([os.path.join(SRC, f) for f in FILES])


def _nT(k):
    return (k + 1) * (k + 2) * (k + 3) // 6


# ----------------------------------------------------------------------------
# tensors

def _points(rng, n, rmin, rmax):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    r = np.exp(rng.uniform(np.log(rmin), np.log(rmax), n))
    return v * r[:, None]


def _mp_call(fx, ns, name, pts, a, ncomp):
    import mpmath
    fx.set_mode("mp")
    try:
        n = len(pts)
        conv = lambda col: np.array([mpmath.mpf(float(t)) for t in col], dtype=object)
        T = np.empty((n, ncomp), dtype=object)
        T[...] = mpmath.mpf(0)
        args = [conv(pts[:, 0]), conv(pts[:, 1]), conv(pts[:, 2])]
        if a is not None:
            args.append(conv(a))
        ns["f_" + name](*args, T[:, : ncomp])
        return np.array([[float(t) for t in row] for row in T])
    finally:
        fx.set_mode("float")


def tensors_job(_):
    fx, tr = _translated()
    out = {}
    rng = np.random.default_rng(20261204)
    # Cnij tables and the recursive undamped tensors
    for bits in (32, 64):
        fx.set_int_bits(bits)
        ns = tr.new()
        pts = _points(np.random.default_rng(7), 24, 0.4, 40.0)
        T = np.zeros((len(pts), _nT(16)), order="F")
        ns["f_tn_recursive"](16, pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), T)
        out["none_rec%d" % bits] = T
        out["cnij%d" % bits] = ns["f_cnij"].a.copy()
        out["none_pts"] = pts
    fx.set_int_bits(32)
    # generated undamped closed forms T0..T12: compiled only where __GNUC__
    # is undefined (src/tensors.F90:12-16); gfortran builds use Tn_recursive
    ns = fx.Translated([os.path.join(SRC, f) for f in FILES[:2]], defines={}).new()
    pts = out["none_pts"]
    gen = np.zeros((len(pts), _nT(12)))
    off = 0
    for k in range(13):
        w = (k + 1) * (k + 2) // 2
        gen[:, off:off + w] = _mp_call(fx, ns, "t%d" % k, pts, None, w)
        off += w
    out["none_gen"] = gen
    # damped kinds: Tn_damp_K(6) in 50 digits and in binary64
    for kind in ("AMOEBA", "THOLE", "ERF"):
        pts = _points(rng, 40, 0.3, 25.0)
        a = rng.uniform(0.09, 0.64, len(pts))
        name = "tn_damp_" + kind.lower()
        ex = np.zeros((len(pts), _nT(6)))
        ns = tr.new()
        for q in range(len(pts)):
            import mpmath
            fx.set_mode("mp")
            try:
                c = lambda v: np.array([mpmath.mpf(float(v))], dtype=object)
                T = np.empty((1, _nT(6)), dtype=object)
                T[...] = mpmath.mpf(0)
                ns["f_" + name](6, c(pts[q, 0]), c(pts[q, 1]), c(pts[q, 2]), c(a[q]), T)
                ex[q] = [float(t) for t in T[0]]
            finally:
                fx.set_mode("float")
        ns = tr.new()
        T64 = np.zeros((len(pts), _nT(6)), order="F")
        ns["f_" + name](6, pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), a.copy(), T64)
        out[kind + "_pts"] = np.column_stack([pts, a])
        out[kind + "_gen"] = ex
        out[kind + "_f64"] = T64
    return out


# ----------------------------------------------------------------------------
# fields

CASES = {
    # name: (system, n_mol or n, box, multipole order, damp, theta, ncrit, p, f, tree, seed)
    "water_none": ("water", 80, 17.0, 2, "", 0.5, 8, 4, 1, True, 11),
    "water_thole": ("water", 70, 16.0, 2, "THOLE", 0.5, 8, 6, 2, True, 12),
    "water_amoeba": ("water", 50, 14.5, 2, "AMOEBA", 0.5, 8, 8, 1, False, 13),
    "uniform_erf": ("uniform", 240, 14.0, 1, "ERF", 0.5, 10, 5, 1, False, 14),
    "uniform_charges": ("uniform", 300, 16.0, 0, "", 0.6, 12, 5, 2, False, 15),
    # octupoles (mdim 20) and field order 3: damped tensors up to order 6
    "uniform_octupole_f3": ("uniform", 120, 12.0, 3, "", 0.5, 10, 5, 3, False, 19),
    "water_octupole_thole_f3": ("water", 30, 11.0, 3, "THOLE", 0.5, 8, 4, 3, False, 20),
    "water_amoeba_f3": ("water", 30, 11.0, 2, "AMOEBA", 0.5, 8, 4, 3, False, 21),
    "uniform_octupole_erf": ("uniform", 90, 11.0, 3, "ERF", 0.5, 10, 4, 1, False, 22),
    # periodic boxes (is_periodic = .true.): particles inside the cell of BOXES[name]
    "periodic_cubic": ("water", 36, 11.0, 2, "", 0.5, 8, 4, 1, False, 16),
    "periodic_triclinic_thole": ("water", 30, 10.5, 2, "THOLE", 0.5, 8, 5, 2, False, 17),
    "periodic_amoeba_p6": ("water", 30, 10.5, 2, "AMOEBA", 0.5, 8, 6, 1, False, 18),
}

# cell vectors as the columns of box_matrix; the triclinic one has
# box(1,2) != box(2,1) and box(1,3) box(3,2) != 0, where the reference's
# volume formula (fmm.F90:963-965) differs from the determinant
BOXES = {
    "periodic_cubic": [[11.0, 0.0, 0.0], [0.0, 11.0, 0.0], [0.0, 0.0, 11.0]],
    "periodic_triclinic_thole": [[10.5, 0.5, 0.3], [1.5, 10.0, 0.4], [0.8, 1.2, 10.2]],
    "periodic_amoeba_p6": [[10.5, 0.0, 0.0], [0.0, 10.5, 0.0], [0.0, 0.0, 10.5]],
}


def _system(spec):
    from fmm_gb300 import systems
    kind, n, box, order, damp = spec[:5]
    seed = spec[10]
    if kind == "water":
        s = systems.water(n, box, order=order, seed=seed)
    else:
        s = systems.uniform_triplets(n, box, order=order, seed=seed)
        rng = np.random.default_rng(seed + 1)
        s["damping_factors"] = rng.uniform(0.3, 0.8, n) if damp == "ERF" else np.zeros(n)
    if damp == "":
        s["damping_factors"] = np.zeros(s["coordinates"].shape[0])
    name = [k for k, v in CASES.items() if v == spec][0]
    if name in BOXES:
        # fractional coordinates wrapped into [0, 1), then the cell
        H = np.array(BOXES[name]).T  # columns are the cell vectors
        u = np.mod(np.linalg.solve(H, np.asarray(s["coordinates"]).T).T, 1.0)
        s["coordinates"] = np.asfortranarray(u @ H.T)
    return s


def _tree_arrays(ns):
    t = ns["f_tree"]
    M = t.f_num_nodes
    cen = np.zeros((M, 3))
    r = np.zeros(M)
    rmax = np.zeros(M)
    depth = np.zeros(M, np.int32)
    parent = np.full(M, -1, np.int32)
    leaf = np.zeros(M, np.int32)
    count = np.zeros(M, np.int32)
    far, near = [], []
    for i in range(1, M + 1):
        nd = t.f_node_list[i].f_node
        cen[i - 1] = nd.f_center.a
        r[i - 1] = nd.f_r
        rmax[i - 1] = nd.f_rmax
        depth[i - 1] = nd.f_depth
        parent[i - 1] = nd.f_parent.f_idx - 1 if nd.f_parent is not None else -1
        leaf[i - 1] = 1 if nd.f_is_terminal else 0
        count[i - 1] = nd.f_nleaf
        for s in nd.f_cell_interactions[1].f_elements.a:
            far.append((i - 1, int(s) - 1))
        for s in nd.f_particle_interactions[1].f_elements.a:
            near.append((i - 1, int(s) - 1))
    return dict(center=cen, r=r, rmax=rmax, depth=depth, parent=parent, leaf=leaf, count=count,
                far=np.array(sorted(far), np.int32).reshape(-1, 2), near=np.array(sorted(near), np.int32).reshape(-1, 2))


def field_job(name):
    fx, tr = _translated()
    spec = CASES[name]
    s = _system(spec)
    _, _, _, _, damp, theta, ncrit, p, f, want_tree, _ = spec
    X = np.asfortranarray(s["coordinates"])
    Mp = np.asfortranarray(s["multipoles"])
    E = np.asfortranarray(s["exclusions"].astype(np.int64))
    d = np.ascontiguousarray(s["damping_factors"])
    n = X.shape[0]
    t0 = time.time()
    ns = tr.new()
    Fd = np.zeros((n, _nT(f)), order="F")
    ns["f_field_direct"](0, X, Mp, E, f, Fd, damp, d)
    ns = tr.new()
    Ff = np.zeros((n, _nT(f)), order="F")
    periodic = name in BOXES
    box = np.asfortranarray(np.array(BOXES[name]).T) if periodic else np.zeros((3, 3), order="F")
    if periodic:
        ns["f_field_fmm"](0, X, Mp, E, theta, ncrit, p, f, Ff, damp, d, 1, box)
        tree = None
    elif want_tree:
        # keep the tree: run the field_fmm steps up to the lists, then the call itself
        ns["f_field_fmm"](0, X, Mp, E, theta, ncrit, p, f, Ff, damp, d, 0, np.zeros((3, 3), order="F"))
        ns2 = tr.new()
        ns2["f_settings"].f_is_periodic = False
        ns2["f_settings"].f_box_matrix.a[...] = 0.0
        ns2["f_octree_build"](ncrit, p, theta, X, Mp)
        ns2["f_build_interaction_lists_fmm"]()
        tree = _tree_arrays(ns2)
    else:
        ns["f_field_fmm"](0, X, Mp, E, theta, ncrit, p, f, Ff, damp, d, 0, np.zeros((3, 3), order="F"))
        tree = None
    out = {name + "_X": X, name + "_M": Mp, name + "_E": s["exclusions"].astype(np.int32), name + "_d": d,
           name + "_box": box,
           name + "_cfg": np.array([theta, ncrit, p, f, DAMP[damp]], dtype=np.float64),
           name + "_direct": Fd, name + "_fmm": Ff}
    if tree:
        for k, v in tree.items():
            out[name + "_tree_" + k] = v
    print("%s: N=%d %.1f s" % (name, n, time.time() - t0), flush=True)
    return out


# ----------------------------------------------------------------------------
# QM/MM helpers (src/fmm.F90:1134-1336).  As shipped they stop in `finalize`
# (clean_node deallocates the interaction lists that these helpers never
# build; gfortran stops at DEALLOCATE of an unallocated array), so their
# outputs are read with that DEALLOCATE skipped; ``qmmm_stops`` records the
# stop of the unmodified code.

def _comps(n):
    return [(kx, ky, k - kx - ky) for k in range(n + 1) for kx in range(k, -1, -1) for ky in range(k - kx, -1, -1)]


def qmmm_job(_):
    fx, tr = _translated()
    from fmm_gb300 import systems
    out = {}
    s = systems.water(90, 15.0, seed=21)
    X = np.asfortranarray(s["coordinates"])
    M = np.asfortranarray(s["multipoles"])
    M3 = np.asfortranarray(np.stack([M, 0.5 * M + 0.01], axis=2))
    rng = np.random.default_rng(22)
    T = np.asfortranarray(X[rng.choice(X.shape[0], 6, replace=False)] + rng.normal(0, 0.3, (6, 3)))
    theta, ncrit, p, f = 0.5, 8, 4, 1
    stops = []
    for name in ("get_boxes", "get_multipoles", "interpolate_electron_fields"):
        try:
            ns = tr.new()
            if name == "get_boxes":
                ns["f_get_boxes"](X, T, theta, ncrit, p, None, None, None)
            elif name == "get_multipoles":
                ns["f_get_multipoles"](0, X, M3, T, theta, ncrit, p, None, None, None)
            else:
                Fx = np.zeros((X.shape[0], _nT(f), 1), order="F")
                ns["f_interpolate_electron_fields"](0, X, np.zeros((1, _nT(p), 1), order="F"),
                                                    np.array([1], dtype=np.int64), theta, ncrit, p, f, Fx)
        except fx.FortranStop as e:
            stops.append("%s: %s" % (name, e))
    fx.set_lenient_dealloc(True)
    try:
        ns = tr.new()
        idx, bc, bi = ns["f_get_boxes"](X, T, theta, ncrit, p, None, None, None)
        ns = tr.new()
        idx2, bc2, bm = ns["f_get_multipoles"](0, X, M3, T, theta, ncrit, p, None, None, None)
        # local expansions at the boxes: random Taylor coefficients that fall
        # off with the order, different per box and per set
        nq = _nT(p)
        nbox = bi.a.shape[0]
        Lx = np.asfortranarray(rng.normal(0, 1.0, (nbox, nq, 2)) * np.array(
            [0.1 ** (sum(c)) for c in _comps(p)])[None, :, None])
        ns = tr.new()
        F = np.zeros((X.shape[0], _nT(f), 2), order="F")
        ns["f_interpolate_electron_fields"](0, X, Lx, bi.a.astype(np.int64), theta, ncrit, p, f, F)
    finally:
        fx.set_lenient_dealloc(False)
    out.update(qmmm_X=X, qmmm_M=M3, qmmm_T=T, qmmm_cfg=np.array([theta, ncrit, p, f]),
               qmmm_idx_near=idx.a.astype(np.int32), qmmm_box_coordinates=bc.a,
               qmmm_box_indices=bi.a.astype(np.int32), qmmm_idx_near_mp=idx2.a.astype(np.int32),
               qmmm_box_coordinates_mp=bc2.a, qmmm_box_multipoles=bm.a, qmmm_local=Lx, qmmm_field=F,
               qmmm_stops=np.array(stops))
    print("qmmm: %d near particles, %d boxes; unmodified: %s" % (idx.a.shape[0], nbox, stops), flush=True)
    return out


def main():
    if not os.path.isdir(SRC):
        raise SystemExit("reference source not found at %s (set FMM_REFERENCE_SRC)" % SRC)
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(8, len(CASES) + 1)) as pool:
        tj = pool.apply_async(tensors_job, (0,))
        qj = pool.apply_async(qmmm_job, (0,))
        fj = pool.map_async(field_job, list(CASES))
        tens = tj.get()
        fields = {}
        for part in fj.get():
            fields.update(part)
        fields.update(qj.get())
    np.savez_compressed(os.path.join(HERE, "ref_tensors.npz"), **tens)
    np.savez_compressed(os.path.join(HERE, "ref_fields.npz"), **fields)
    print("wrote ref_tensors.npz (%d arrays), ref_fields.npz (%d arrays)" % (len(tens), len(fields)))


if __name__ == "__main__":
    main()

"""The allocation-free direct sum (fmm_field_direct_targets_noalloc) against
the allocating entry point (fmm_field_direct_targets_device).

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.  The allocation-free entry
point exists for callers that cannot let the library allocate device memory
(their memory manager owns the device, or they must avoid the synchronisation
an allocation can cause); its only scratch is a fixed static device array, so
the caller provides every input and output buffer, as done here with torch.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _setup(n_mol=1000, ntgt=700, seed=21):
    torch = pytest.importorskip("torch")
    from fmm_gb300 import systems
    s = systems.water(n_mol, 35.0, seed=seed)
    n = 3 * n_mol
    dev = torch.device("cuda", 0)
    col = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).T).reshape(-1)).to(dev)
    buf = dict(X=col(s["coordinates"]), M=col(s["multipoles"]), E=col(s["exclusions"]),
               D=torch.from_numpy(s["damping_factors"].copy()).to(dev))
    rng = np.random.default_rng(seed)
    tgt = np.sort(rng.choice(n, ntgt, replace=False)).astype(np.int64)
    buf["T"] = torch.from_numpy(tgt).to(dev)
    return torch, n, buf


def _call(L, fn, n, buf, ntgt, out, f=1, damp=b"AMOEBA", excl_mode=0, targets=None):
    from fmm_gb300 import _lib
    o = _lib.FmmOpts()
    o.version = 1
    o.excl_mode = excl_mode
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    T = targets if targets is not None else buf["T"]
    return getattr(L, fn)(n, p(buf["X"]), 10, p(buf["M"]), 3, p(buf["E"]), ntgt, p(T), f, p(out), damp, len(damp),
                          p(buf["D"]), ctypes.byref(o))


@pytest.mark.parametrize("excl_mode,damp,f", [(0, b"AMOEBA", 1), (1, b"THOLE", 2), (0, b"", 1)])
def test_noalloc_matches_allocating_entry_point(excl_mode, damp, f):
    from fmm_gb300 import _lib
    L = _lib.lib()
    torch, n, buf = _setup()
    ntgt = buf["T"].numel()
    nf = (f + 1) * (f + 2) * (f + 3) // 6
    ref = torch.empty(ntgt * nf, dtype=torch.float64, device="cuda")
    assert _call(L, "fmm_field_direct_targets_device", n, buf, ntgt, ref, f, damp, excl_mode) == 0
    torch.cuda.synchronize()
    R = ref.cpu().numpy()
    for _ in range(2):  # two calls in a row share the static scratch
        out = torch.full((ntgt * nf,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(L, "fmm_field_direct_targets_noalloc", n, buf, ntgt, out, f, damp, excl_mode) == 0
        torch.cuda.synchronize()
        G = out.cpu().numpy()
        assert np.all(np.isfinite(G))
        assert np.linalg.norm(G - R) <= TOL * np.linalg.norm(R)


def test_noalloc_matches_oracle_rows():
    """The allocation-free entry point against the CPU oracle's direct sum
    (the reference's field_direct semantics, src/fmm.F90:749-824), row by row
    at the sampled targets, in both exclusion modes."""
    import oracle
    from fmm_gb300 import _lib, systems
    L = _lib.lib()
    torch, n, buf = _setup(n_mol=400, ntgt=300, seed=5)
    s = systems.water(400, 35.0, seed=5)
    tgt = buf["T"].cpu().numpy()
    for excl_mode, mode in ((0, "ref"), (1, "mask")):
        O = oracle.field_direct(0, s["coordinates"], s["multipoles"], s["exclusions"], 1, "AMOEBA",
                                s["damping_factors"], excl_mode=mode)[tgt]
        for _ in range(2):
            out = torch.full((len(tgt) * 4,), float("nan"), dtype=torch.float64, device="cuda")
            assert _call(L, "fmm_field_direct_targets_noalloc", n, buf, len(tgt), out, 1, b"AMOEBA",
                         excl_mode) == 0
            torch.cuda.synchronize()
            G = out.cpu().numpy().reshape(4, -1).T
            # AMOEBA has no potential (T0 = 0 in the reference): field columns only
            assert np.linalg.norm(G[:, 1:] - O[:, 1:]) <= TOL * np.linalg.norm(O[:, 1:])


def test_noalloc_at_the_size_limit():
    """Exactly FMM_NOALLOC_MAX_VALUES outputs (field order 0: one value per
    target, targets repeated), where the source split is limited by the
    static scratch, against the allocating entry point."""
    from fmm_gb300 import _lib
    L = _lib.lib()
    torch, n, buf = _setup(n_mol=1000, ntgt=10, seed=8)
    ntgt = 524256
    rng = np.random.default_rng(8)
    T = torch.from_numpy(rng.integers(0, n, ntgt).astype(np.int64)).to("cuda")
    ref = torch.empty(ntgt, dtype=torch.float64, device="cuda")
    assert _call(L, "fmm_field_direct_targets_device", n, buf, ntgt, ref, 0, b"THOLE", 0, targets=T) == 0
    torch.cuda.synchronize()
    R = ref.cpu().numpy()
    for _ in range(2):
        out = torch.full((ntgt,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(L, "fmm_field_direct_targets_noalloc", n, buf, ntgt, out, 0, b"THOLE", 0, targets=T) == 0
        torch.cuda.synchronize()
        G = out.cpu().numpy()
        assert np.all(np.isfinite(G))
        assert np.linalg.norm(G - R) <= TOL * np.linalg.norm(R)


def test_noalloc_rejects_bad_exclusion_on_any_row():
    """An exclusion entry outside 0..n is rejected as by the allocating entry
    point, also when it sits in a row that is not one of the targets."""
    from fmm_gb300 import _lib
    L = _lib.lib()
    torch, n, buf = _setup(n_mol=300, ntgt=20, seed=9)
    tgt = set(buf["T"].cpu().numpy().tolist())
    row = next(i for i in range(n) if i not in tgt)
    E = buf["E"].clone()
    E[2 * n + row] = n + 1  # third column of a non-target row
    bad = dict(buf, E=E)
    ntgt = buf["T"].numel()
    out = torch.empty(ntgt * 4, dtype=torch.float64, device="cuda")
    assert _call(L, "fmm_field_direct_targets_device", n, bad, ntgt, out) == _lib.FMM_EINVAL
    assert _call(L, "fmm_field_direct_targets_noalloc", n, bad, ntgt, out) == _lib.FMM_EINVAL
    # and a good call right after still works
    assert _call(L, "fmm_field_direct_targets_noalloc", n, buf, ntgt, out) == 0


def test_noalloc_rejects_oversized_and_bad_targets():
    from fmm_gb300 import _lib
    L = _lib.lib()
    torch, n, buf = _setup(n_mol=300, ntgt=200)
    ntgt = 524256 // 4 + 1  # field_order 1: 4 values per target
    big_t = torch.zeros(ntgt, dtype=torch.int64, device="cuda")
    out = torch.empty(ntgt * 4, dtype=torch.float64, device="cuda")
    assert _call(L, "fmm_field_direct_targets_noalloc", n, buf, ntgt, out, targets=big_t) == _lib.FMM_EINVAL
    bad_t = torch.tensor([0, 1, n], dtype=torch.int64, device="cuda")
    out = torch.empty(3 * 4, dtype=torch.float64, device="cuda")
    assert _call(L, "fmm_field_direct_targets_noalloc", n, buf, 3, out, targets=bad_t) == _lib.FMM_EINVAL

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

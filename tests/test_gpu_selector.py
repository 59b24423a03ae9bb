"""Selector network kernels against the numpy reference (oracle/mlp.py)."""
import ctypes

import numpy as np
import pytest

from oracle import mlp as ref

pytestmark = pytest.mark.gpu


def _L():
    from fmm_gb300 import _lib
    L = _lib.lib()
    L.fmm_mlp_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    L.fmm_mlp_grad.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                               ctypes.c_void_p]
    L.fmm_mlp_param_count.restype = ctypes.c_int
    return L


def _data(n=300, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, ref.IN)).astype(np.float32) * 3 + 1
    Y = rng.normal(size=(n, ref.OUT)).astype(np.float32)
    p = ref.init_params(X, seed)
    return X, Y, p


def test_param_layout_matches():
    assert _L().fmm_mlp_param_count() == ref.offsets()["total"]


def test_forward_matches_numpy():
    L = _L()
    X, Y, p = _data()
    out = np.zeros((X.shape[0], ref.OUT), dtype=np.float32)
    assert L.fmm_mlp_forward(p.ctypes.data, X.ctypes.data, X.shape[0], out.ctypes.data) == 0
    yref, _ = ref.forward(p.astype(np.float64), X.astype(np.float64))
    # inference runs on the tensor cores with FP16 operands (FP32
    # accumulation): outputs (log10 errors) agree to ~1e-3 relative, far below
    # the network's own prediction error (~0.3 in log10)
    assert np.max(np.abs(out - yref)) <= 1e-2 * max(1.0, np.max(np.abs(yref)))


def test_gradient_matches_numpy():
    L = _L()
    X, Y, p = _data(n=256, seed=1)  # a multiple of the 64-sample training block
    g = np.zeros(ref.offsets()["total"], dtype=np.float32)
    loss = ctypes.c_float(0)
    assert L.fmm_mlp_grad(p.ctypes.data, X.ctypes.data, Y.ctypes.data, X.shape[0], g.ctypes.data,
                          ctypes.byref(loss)) == 0
    lref, gref = ref.loss_and_grad(p.astype(np.float64), X.astype(np.float64), Y.astype(np.float64))
    assert abs(loss.value - lref) <= 1e-5 * lref
    o = ref.offsets()
    for name in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"):
        a, n = o[name]
        d = np.abs(g[a:a + n] - gref[a:a + n]).max()
        assert d <= 1e-4 * max(1e-3, np.abs(gref[a:a + n]).max()), name

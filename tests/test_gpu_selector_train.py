"""Training pieces of the learned expansion-order selector on the GPU:
the Adam update of fmm_mlp_train against numpy, loss decrease, and the
collector's labels (log10 RMS field error of a far pair's expansion truncated
at order q) against a CPU evaluation of the same truncated Taylor expansion
built from the oracle's interaction tensors."""
import ctypes

import numpy as np
import pytest

import oracle
from fmm_gb300 import _lib, selector_train, systems

pytestmark = pytest.mark.gpu

IN, OUT, QMIN = selector_train.IN, selector_train.OUT, 2


def _lib_mlp():
    L = _lib.lib()
    L.fmm_mlp_grad.restype = ctypes.c_int
    L.fmm_mlp_grad.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                               ctypes.c_void_p]
    L.fmm_mlp_param_count.restype = ctypes.c_int
    return L


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, (n, IN)).astype(np.float32)
    W = rng.normal(0, 0.3, (IN, OUT)).astype(np.float32)
    Y = (np.tanh(X @ W) - 0.2 * np.arange(OUT)[None, :]).astype(np.float32)
    return X, Y


def test_one_adam_step_matches_numpy():
    L = _lib_mlp()
    n = 256
    X, Y = _data(n, 1)
    p0 = selector_train.init_params(X, seed=3)
    assert p0.size == L.fmm_mlp_param_count()
    g = np.zeros_like(p0)
    loss = ctypes.c_float(0)
    _lib.check(L.fmm_mlp_grad(p0.ctypes.data, X.ctypes.data, Y.ctypes.data, n, g.ctypes.data, ctypes.byref(loss)),
               "fmm_mlp_grad")
    lr = 1e-2
    p1, losses = selector_train.train(X, Y, epochs=1, batch=n, lr=lr, seed=3)
    # one epoch of one batch: learning rate 0.1 lr (the final tenth of the
    # schedule), bias-corrected first step = -lr g / (|g| + 1e-8)
    lr_e = 0.1 * lr
    off_w1 = 2 * IN
    assert np.array_equal(p1[:off_w1], p0[:off_w1])  # normalisation untouched
    step = p1[off_w1:] - p0[off_w1:]
    gg = g[off_w1:]
    assert np.all(np.abs(step) <= lr_e * (1 + 1e-5) + 1e-7)
    big = np.abs(gg) > 1e-5
    assert big.mean() > 0.5
    expect = -lr_e * gg[big] / (np.abs(gg[big]) + 1e-8)
    assert np.max(np.abs(step[big] - expect)) <= 1e-3 * lr_e + 1e-7
    assert abs(losses[0] - loss.value) <= 1e-4 * abs(loss.value)


def test_training_lowers_the_loss():
    X, Y = _data(4096, 2)
    _, losses = selector_train.train(X, Y, epochs=30, batch=256, lr=2e-3, seed=0)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.2 * losses[0]


def _comps(n):
    return [(kx, ky, k - kx - ky) for k in range(n + 1) for kx in range(k, -1, -1) for ky in range(k - kx, -1, -1)]


def _truncated_error(Xs, qs, Xt, ci, cj, q, Tfun, cidx):
    """RMS over targets of |F_q - F_exact| for charges qs at Xs seen from
    targets Xt, source moments about cj and local expansion about ci both
    truncated at order q (field = gradient of the potential)."""
    from math import factorial
    comps = _comps(2 * q)
    a = Xs - cj
    # M_s = sum_p q_p (-a)^s / s!, |s| <= q
    Ms = {}
    for s in _comps(q):
        Ms[s] = np.sum(qs * np.prod([(-a[:, c]) ** s[c] / factorial(s[c]) for c in range(3)], axis=0))
    T = Tfun(ci - cj, 2 * q)
    L = {}
    for g in _comps(q):
        L[g] = sum(Ms[s] * T[cidx[(s[0] + g[0], s[1] + g[1], s[2] + g[2])]] for s in Ms)
    err2 = 0.0
    for x in Xt:
        d = x - ci
        F = np.zeros(3)
        for w in _comps(q - 1):
            dw = np.prod([d[c] ** w[c] / factorial(w[c]) for c in range(3)])
            for u in range(3):
                gu = list(w)
                gu[u] += 1
                F[u] += L[tuple(gu)] * dw
        r = x - Xs
        rn = np.linalg.norm(r, axis=1)
        Fx = np.array([np.sum(qs * T1) for T1 in (-(r / rn[:, None] ** 3)).T])
        err2 += np.sum((F - Fx) ** 2)
    assert len(comps) > 0
    return np.sqrt(err2 / len(Xt))


def test_collector_labels_match_cpu_truncation():
    s = systems.uniform_triplets(3000, 30.0, order=0, seed=5)
    X = np.asfortranarray(s["coordinates"])
    qch = np.asfortranarray(s["multipoles"][:, :1])
    ncrit, theta, maxp = 8, 0.5, 400
    L = _lib.lib()
    L.fmm_selector_collect.restype = ctypes.c_int
    L.fmm_selector_collect.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_uint64,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                       ctypes.c_void_p]
    F = np.zeros((maxp, IN), np.float32)
    Y = np.zeros((maxp, OUT), np.float32)
    pairs = np.zeros((maxp, 2), np.int32)
    npairs = ctypes.c_int(0)
    _lib.check(L.fmm_selector_collect(X.shape[0], X.ctypes.data, 1, qch.ctypes.data, None, ncrit, theta, maxp, 9,
                                      F.ctypes.data, Y.ctypes.data, ctypes.byref(npairs), pairs.ctypes.data),
               "fmm_selector_collect")
    npr = npairs.value
    assert npr == maxp
    assert np.all(np.isfinite(F[:npr])) and np.all(np.isfinite(Y[:npr]))
    t = oracle.tree(X, ncrit, theta, centroid="blocked")
    far = {(int(a), int(b)) for a, b in t["far"]}
    assert all((int(a), int(b)) in far for a, b in pairs[:npr])
    # the particles of each node: leaves, then ancestors by the parent array
    M = t["center"].shape[0]
    members = [[] for _ in range(M)]
    for k, lf in enumerate(t["leaf_of"]):
        node = int(lf)
        while node >= 0:
            members[node].append(k)
            node = int(t["parent"][node])
    cidx = {c: k for k, c in enumerate(_comps(16))}

    def Tfun(R, n):
        T = oracle.tensors(n, np.array([R[0]]), np.array([R[1]]), np.array([R[2]]), "", coef="exact")[0]
        # plain derivatives of 1/r: T_x = -x / r^3
        assert abs(T[1] + R[0] / np.linalg.norm(R) ** 3) <= 1e-12 * abs(T[1]) + 1e-300
        return T

    checked = 0
    for k in range(npr):
        i, j = (int(v) for v in pairs[k])
        tgt = members[i]
        if not t["is_leaf"][i] or len(tgt) > 8:
            continue
        src = np.array(members[j])
        for q in range(QMIN, 9):
            e = _truncated_error(X[src], qch[src, 0], X[tgt], t["center"][i], t["center"][j], q, Tfun, cidx)
            ref = np.log10(max(e, 1e-14))
            if ref < -11.5:
                continue
            assert abs(Y[k, q - QMIN] - ref) <= 2e-3, (i, j, q, Y[k, q - QMIN], ref)
            checked += 1
        if checked >= 120:
            break
    assert checked >= 60

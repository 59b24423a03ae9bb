"""Trains the expansion-order selector on the GPU.

    python -m fmm_gb300.selector_train [--systems 50] [--blob-systems 25] [--n-mol 33334]
                                       [--out fmm_gb300/data/selector_v2]

For each of `systems` seeded water-like systems (N = 3 x n_mol particles at
the density of the 1M benchmark system, AMOEBA damping factors) and
`blob_systems` clustered ones (Gaussian blobs as the 2M clustered benchmark
system, scaled to the same N at its density) far pairs are
sampled from the far lists of the reference acceptance test at several theta
values, and the library measures each pair's M2L + L2P field error at
expansion orders 2..12 against the FP64 direct sum over the source cell
(fmm_selector_collect).  The network (fmm_mlp_train: fused forward/backward
kernels and Adam, all on the GPU) learns log10 of those errors from the pair
features.  Weights are written as raw float32 (<out>.bin) with a JSON header
(<out>.json).
"""
import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from fmm_gb300 import _lib, systems  # noqa: E402

IN, OUT = 17, 11
DEFAULT_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "selector_v2")


def make_training_system(kind, n_mol, seed):
    """water: water-like triplets at the density of the 1M benchmark system;
    blobs: the clustered benchmark system's kind (64 Gaussian blobs) scaled to
    3 n_mol particles at its density."""
    if kind == "water":
        box = 270.0 * (n_mol / 333_333) ** (1.0 / 3.0)
        return systems.water(n_mol, box, seed=seed)
    n = 3 * n_mol
    sc = (n / 2_000_000) ** (1.0 / 3.0)
    return systems.blobs(n=n, box=600.0 * sc, sigma_range=(5.0 * sc, 30.0 * sc), seed=seed)


def collect(n_systems, n_mol, thetas, pairs_per_theta, ncrit=64, seed0=1000, kind="water"):
    L = _lib.lib()
    L.fmm_selector_collect.restype = ctypes.c_int
    L.fmm_selector_collect.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    Xs, Ys = [], []
    for k in range(n_systems):
        s = make_training_system(kind, n_mol, seed0 + k)
        Xc = np.asfortranarray(s["coordinates"])
        Mc = np.asfortranarray(s["multipoles"])
        d = np.ascontiguousarray(s["damping_factors"])
        for t in thetas:
            F = np.zeros((pairs_per_theta, IN), dtype=np.float32)
            Y = np.zeros((pairs_per_theta, OUT), dtype=np.float32)
            npairs = ctypes.c_int(0)
            st = L.fmm_selector_collect(Xc.shape[0], Xc.ctypes.data, Mc.shape[1], Mc.ctypes.data, d.ctypes.data, ncrit,
                                        float(t), pairs_per_theta, seed0 + 7 * k, F.ctypes.data, Y.ctypes.data,
                                        ctypes.byref(npairs), None)
            _lib.check(st, "fmm_selector_collect")
            Xs.append(F[:npairs.value])
            Ys.append(Y[:npairs.value])
    return np.concatenate(Xs), np.concatenate(Ys)


H = 64


def init_params(X, seed=0):
    """Input normalisation from the training features, He-initialised weights,
    zero biases (layout of fmm_gb300/csrc/mlp.cuh)."""
    rng = np.random.default_rng(seed)
    sizes = [IN, IN, H * IN, H, H * H, H, H * H, H, OUT * H, OUT]
    p = np.zeros(sum(sizes), dtype=np.float32)
    std = X.std(0)
    std[std < 1e-6] = 1.0
    p[0:IN] = X.mean(0)
    p[IN:2 * IN] = 1.0 / std
    off = 2 * IN
    for size, fan_in, is_w in zip(sizes[2:], (IN, 0, H, 0, H, 0, H, 0), (1, 0, 1, 0, 1, 0, 1, 0)):
        if is_w:
            p[off:off + size] = rng.normal(0.0, np.sqrt(2.0 / fan_in), size)
        off += size
    return p


def train(X, Y, epochs=40, batch=256, lr=2e-3, seed=0):
    L = _lib.lib()
    L.fmm_mlp_train.restype = ctypes.c_int
    L.fmm_mlp_train.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                ctypes.c_int, ctypes.c_float, ctypes.c_uint64, ctypes.c_void_p]
    p = init_params(X, seed)
    losses = np.zeros(epochs, dtype=np.float32)
    Xc = np.ascontiguousarray(X, dtype=np.float32)
    Yc = np.ascontiguousarray(Y, dtype=np.float32)
    st = L.fmm_mlp_train(p.ctypes.data, Xc.ctypes.data, Yc.ctypes.data, Xc.shape[0], epochs, batch, lr, seed,
                         losses.ctypes.data)
    _lib.check(st, "fmm_mlp_train")
    return p, losses


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=50)
    ap.add_argument("--blob-systems", type=int, default=25)
    ap.add_argument("--n-mol", type=int, default=33_334)
    ap.add_argument("--pairs", type=int, default=1500, help="sampled far pairs per system and theta")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--out", default=DEFAULT_OUT)
    args = ap.parse_args()
    thetas = (0.25, 0.35, 0.5, 0.7)
    t0 = time.time()
    X, Y = collect(args.systems, args.n_mol, thetas, args.pairs)
    if args.blob_systems > 0:
        Xb, Yb = collect(args.blob_systems, args.n_mol, thetas, args.pairs, seed0=2000, kind="blobs")
        X, Y = np.concatenate([X, Xb]), np.concatenate([Y, Yb])
    t1 = time.time()
    rng = np.random.default_rng(0)
    perm = rng.permutation(X.shape[0])
    nval = X.shape[0] // 10
    Xv, Yv = X[perm[:nval]], Y[perm[:nval]]
    Xt, Yt = X[perm[nval:]], Y[perm[nval:]]
    p, losses = train(Xt, Yt, epochs=args.epochs)
    t2 = time.time()
    # validation error of the log10 predictions
    L = _lib.lib()
    L.fmm_mlp_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    Yp = np.zeros_like(Yv)
    _lib.check(L.fmm_mlp_forward(p.ctypes.data, np.ascontiguousarray(Xv).ctypes.data, Xv.shape[0], Yp.ctypes.data),
               "fmm_mlp_forward")
    res = Yp - Yv
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    p.astype("<f4").tofile(args.out + ".bin")
    meta = {
        "format": "fmm_gb300 selector weights v1 (float32 little-endian)",
        "layout": "mean[17] istd[17] W1[64][17] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[11][64] b4[11]",
        "outputs": "log10 RMS field error of the pair's M2L+L2P contribution at expansion orders 2..12",
        "features": ["rho=sqrt3(r_i+r_j)/R", "log2(r_j/r_i)", "log2(count_i)"] +
                    ["log10(|w^(%d)_j|/R^%d)" % (k, k + 2) for k in range(13)] + ["min(dmin_i dmin_j R,30)/30"],
        "training": {"systems": args.systems, "blob_systems": args.blob_systems,
                     "particles_per_system": 3 * args.n_mol, "thetas": thetas,
                     "pairs_per_system_theta": args.pairs, "samples": int(X.shape[0]), "epochs": args.epochs,
                     "train_loss_last": float(losses[-1]), "collect_s": round(t1 - t0, 1),
                     "train_s": round(t2 - t1, 1)},
        "validation": {"samples": int(nval), "rmse_log10": float(np.sqrt(np.mean(res ** 2))),
                       "p95_abs_log10": float(np.quantile(np.abs(res), 0.95)),
                       "max_abs_log10": float(np.abs(res).max())},
        "losses": [float(v) for v in losses],
    }
    json.dump(meta, open(args.out + ".json", "w"), indent=1)
    print(json.dumps({k: meta[k] for k in ("training", "validation")}))


if __name__ == "__main__":
    main()

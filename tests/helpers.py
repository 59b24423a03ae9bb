"""Shared helpers of the test suite."""
import numpy as np


def rel_err(F, G, cols=None):
    """Global relative error ||F - G|| / ||G|| over the selected columns."""
    F = np.asarray(F)
    G = np.asarray(G)
    if cols is not None:
        F = F[:, cols]
        G = G[:, cols]
    return float(np.linalg.norm(F - G) / max(np.linalg.norm(G), 1e-300))


def per_target_rel(F, G, cols):
    """Per-target relative errors ||F_i - G_i|| / ||G_i|| over columns `cols`."""
    d = np.linalg.norm(np.asarray(F)[:, cols] - np.asarray(G)[:, cols], axis=1)
    g = np.linalg.norm(np.asarray(G)[:, cols], axis=1)
    return d / np.maximum(g, 1e-300)


def small_system(n=600, box=20.0, order=2, seed=0, damp=""):
    from fmm_gb300 import systems
    s = systems.uniform_triplets(n, box, order=order, seed=seed)
    rng = np.random.default_rng(seed + 100)
    if damp == "ERF":
        s["damping_factors"] = rng.uniform(0.3, 0.8, n)
    elif damp:
        alpha = rng.uniform(1.0, 10.0, n)
        s["damping_factors"] = np.sqrt(0.39) / alpha ** (1.0 / 6.0)
    return s

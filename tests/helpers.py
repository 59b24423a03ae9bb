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


def potential_up_to_constant(F, G):
    """Potential column of a periodic result against another: the part that
    varies over the particles (relative to the column's full magnitude) and
    the relative difference of the constants.  The reference's lattice sum
    leaves the potential out of its convergence test (src/fmm.F90:950), so
    the potential carries a constant that, when the sum does not converge, is
    dominated by rounding; only the varying part is then well-conditioned."""
    f = np.asarray(F)[:, 0]
    g = np.asarray(G)[:, 0]
    var = float(np.linalg.norm((f - f.mean()) - (g - g.mean())) / max(np.linalg.norm(g), 1e-300))
    const = float(abs(f.mean() - g.mean()) / max(abs(g.mean()), 1e-300))
    return var, const

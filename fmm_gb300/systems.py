"""Seeded synthetic particle systems with the shapes of the benchmark cases.

Every generator returns a dict with Fortran-ordered arrays in the layout the
reference's ``field_fmm`` / ``field_direct`` take (src/fmm.F90:1338-1371):
``coordinates`` (N, 3) float64, ``multipoles`` (N, dim) float64 in the packed
alphabetical order (q; x, y, z; xx, xy, xz, yy, yz, zz), ``exclusions``
(N, width) int32, 1-based and zero-padded, and ``damping_factors`` (N,).

No public dataset is involved: these stand in for the molecular systems the
library is used on (water-like triplets, uniform and clustered point sets).
"""
import math

import numpy as np

__all__ = ["uniform_triplets", "water", "batched_uniform", "blobs", "haar_rotations"]


def _multipoles(rng, n, order, groups):
    dim = (order + 1) * (order + 2) * (order + 3) // 6
    M = np.zeros((n, dim), order="F")
    q = rng.normal(0.0, 0.5, n)
    for g in groups:
        q[g] -= q[g].mean()
    M[:, 0] = q
    if order >= 1:
        M[:, 1:4] = rng.normal(0.0, 0.1, (n, 3))
    if order >= 2:
        M[:, 4:10] = rng.normal(0.0, 0.05, (n, 6))
    if order >= 3:
        M[:, 10:] = rng.normal(0.0, 0.02, (n, dim - 10))
    return M


def _exclusions(n, groups, width):
    E = np.zeros((n, width), dtype=np.int32, order="F")
    for g in groups:
        for k, i in enumerate(g):
            E[i, : len(g)] = np.asarray(g, dtype=np.int32) + 1
    return E


def _triplet_groups(n):
    return [list(range(s, min(s + 3, n))) for s in range(0, n, 3)]


def uniform_triplets(n=4096, box=40.0, order=2, seed=0):
    """N points uniform in [0, box)^3, grouped into consecutive triplets that
    exclude each other (self included, width 3); charges neutral per group."""
    rng = np.random.default_rng(seed)
    X = np.asfortranarray(rng.uniform(0.0, box, (n, 3)))
    groups = _triplet_groups(n)
    return dict(coordinates=X, multipoles=_multipoles(rng, n, order, groups),
                exclusions=_exclusions(n, groups, 3), damping_factors=np.zeros(n), groups=groups)


def haar_rotations(rng, k):
    """k Haar-random rotation matrices (QR of Gaussian matrices, sign-fixed)."""
    A = rng.normal(size=(k, 3, 3))
    Q, R = np.linalg.qr(A)
    s = np.sign(np.diagonal(R, axis1=1, axis2=2))
    Q = Q * s[:, None, :]
    det = np.linalg.det(Q)
    Q[det < 0, :, 0] *= -1.0
    return Q


def water(n_mol, box, order=2, seed=0, alpha_range=(1.0, 10.0)):
    """Water-like triplets: O uniform in [0, box)^3, two H at 1.8 bohr with an
    H-O-H angle of 104.5 degrees, randomly oriented.  Damping factors
    sqrt(0.39) / alpha^(1/6) with alpha ~ U(alpha_range)."""
    rng = np.random.default_rng(seed)
    O = rng.uniform(0.0, box, (n_mol, 3))
    half = math.radians(104.5) / 2.0
    h1 = np.array([1.8 * math.sin(half), 0.0, 1.8 * math.cos(half)])
    h2 = np.array([-1.8 * math.sin(half), 0.0, 1.8 * math.cos(half)])
    Rm = haar_rotations(rng, n_mol)
    H1 = O + Rm @ h1
    H2 = O + Rm @ h2
    n = 3 * n_mol
    X = np.empty((n, 3))
    X[0::3] = O
    X[1::3] = H1
    X[2::3] = H2
    groups = _triplet_groups(n)
    alpha = rng.uniform(alpha_range[0], alpha_range[1], n)
    d = math.sqrt(0.39) / alpha ** (1.0 / 6.0)
    return dict(coordinates=np.asfortranarray(X), multipoles=_multipoles(rng, n, order, groups),
                exclusions=_exclusions(n, groups, 3), damping_factors=d, groups=groups)


def batched_uniform(n_systems=512, nmin=1000, nmax=65536, density=0.1, order=1, seed=0, erf_range=(0.3, 0.8)):
    """Independent uniform systems with N log-uniform in [nmin, nmax], each in a
    cube at the given density; erf damping factors ~ U(erf_range).  Returns a
    list of per-system dicts (exclusions: self only)."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(math.log(nmin), math.log(nmax), n_systems))).astype(np.int64)
    out = []
    for k, n in enumerate(sizes):
        n = int(n)
        box = (n / density) ** (1.0 / 3.0)
        X = np.asfortranarray(rng.uniform(0.0, box, (n, 3)))
        groups = [[i] for i in range(n)]
        M = _multipoles(rng, n, order, [list(range(n))])
        E = np.asfortranarray(np.arange(1, n + 1, dtype=np.int32).reshape(n, 1))
        d = rng.uniform(erf_range[0], erf_range[1], n)
        out.append(dict(coordinates=X, multipoles=M, exclusions=E, damping_factors=d))
    return out


def blobs(n=2_000_000, n_blobs=64, box=600.0, sigma_range=(5.0, 30.0), order=2, seed=0):
    """Clustered particles: Gaussian blobs with sigma ~ U(sigma_range), centres
    uniform in [0, box)^3, blob weights Dirichlet(1); consecutive triplets
    exclude each other; AMOEBA-style damping factors as in ``water``."""
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.ones(n_blobs))
    counts = rng.multinomial(n, w)
    cen = rng.uniform(0.0, box, (n_blobs, 3))
    sig = rng.uniform(sigma_range[0], sigma_range[1], n_blobs)
    X = np.concatenate([cen[b] + sig[b] * rng.normal(size=(counts[b], 3)) for b in range(n_blobs)])
    perm = rng.permutation(n)
    X = np.asfortranarray(X[perm])
    groups = _triplet_groups(n)
    alpha = rng.uniform(1.0, 10.0, n)
    d = math.sqrt(0.39) / alpha ** (1.0 / 6.0)
    return dict(coordinates=X, multipoles=_multipoles(rng, n, order, groups),
                exclusions=_exclusions(n, groups, 3), damping_factors=d, groups=groups)

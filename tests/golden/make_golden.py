"""Generates tensors_sympy.npz: Cartesian interaction tensors of the four
kernels of the reference (src/tensors_recursive.F90, src/tensors_damped_*.F90)
by symbolic differentiation with sympy, evaluated at 30 significant digits.

Kernels (a = product of the two particles' damping factors):
  ""      phi = 1/r
  THOLE   phi = (1 - (1 + a r / 2) exp(-a r)) / r
  ERF     phi = erf(sqrt(a) r) / r
  AMOEBA  T0 = 0, T_x = -(1 - exp(-a^3 r^3)) x / r^3 (and y, z); higher
          orders are derivatives of these.
T[k] for packed index k (alphabetical: x descending, then y descending).

Run:  python tests/golden/make_golden.py
"""
import os

import numpy as np
import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
NMAX = 6


def comps(nmax):
    out = []
    for n in range(nmax + 1):
        for kx in range(n, -1, -1):
            for ky in range(n - kx, -1, -1):
                out.append((kx, ky, n - kx - ky))
    return out


def main():
    x, y, z, a = sp.symbols("x y z a", real=True)
    r = sp.sqrt(x * x + y * y + z * z)
    phis = {"": 1 / r, "THOLE": (1 - (1 + a * r / 2) * sp.exp(-a * r)) / r, "ERF": sp.erf(sp.sqrt(a) * r) / r}
    g1 = -(1 - sp.exp(-a ** 3 * r ** 3)) / r ** 3
    rng = np.random.default_rng(2024)
    pts = []
    for scale in (0.4, 1.5, 3.0, 7.0, 15.0):
        for _ in range(2):
            v = rng.normal(size=3)
            v = v / np.linalg.norm(v) * scale
            pts.append((float(v[0]), float(v[1]), float(v[2])))
    avals = [0.2, 0.39, 0.64]
    out = {}
    for name in ["", "THOLE", "ERF", "AMOEBA"]:
        rows = []
        for (px, py, pz) in pts:
            for av in (avals if name else [0.0]):
                vals = []
                sub = {x: sp.Rational(repr(px)), y: sp.Rational(repr(py)), z: sp.Rational(repr(pz)),
                       a: sp.Rational(repr(av))}
                for (kx, ky, kz) in comps(NMAX):
                    if name == "AMOEBA":
                        if kx + ky + kz == 0:
                            vals.append(0.0)
                            continue
                        if kx > 0:
                            e = sp.diff(g1 * x, x, kx - 1, y, ky, z, kz)
                        elif ky > 0:
                            e = sp.diff(g1 * y, y, ky - 1, z, kz)
                        else:
                            e = sp.diff(g1 * z, z, kz - 1)
                    else:
                        e = phis[name]
                        if kx:
                            e = sp.diff(e, x, kx)
                        if ky:
                            e = sp.diff(e, y, ky)
                        if kz:
                            e = sp.diff(e, z, kz)
                    vals.append(float(sp.N(e.subs(sub), 30)))
                rows.append([px, py, pz, av] + vals)
        out[name or "NONE"] = np.array(rows)
        print(name or "NONE", out[name or "NONE"].shape, flush=True)
    np.savez_compressed(os.path.join(HERE, "tensors_sympy.npz"), **out)


if __name__ == "__main__":
    main()

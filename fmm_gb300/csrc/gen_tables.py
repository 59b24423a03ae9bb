"""Generates series_tables.h: exact Taylor coefficients for the damped radial
derivative functions used by the near-field and direct-sum kernels.

For a radial kernel phi(r) define g_j(r) = (r^-1 d/dr)^j phi(r).  The damped
kernels of the reference (src/tensors_damped_{thole,amoeba}.F90) have
    g_j(r) = N_j(x) / r^(2j+1)
with a numerator N_j that tends to zero at small argument, where the closed
form cancels catastrophically.  There the kernels evaluate N_j from its
Taylor series, whose coefficients are produced here with exact rational
arithmetic (so coefficients that vanish are exactly zero):

  THOLE  phi = (1 - (1 + a r / 2) e^{-a r}) / r,  x = a r
         N_j(x) = sum_k c_k P_j(k-1) x^k,  c_k = (-1)^(k+1) (1 - k/2) / k!
  AMOEBA g_1 = -(1 - e^{-u}) / r^3,  u = (a r)^3,  g_0 = 0
         N_j(u) = sum_k s_k P_{j-1}(3k-3) u^k,  s_k = (-1)^k / k!
where P_j(m) = m (m-2) (m-4) ... (m-2j+2) comes from (r^-1 d/dr)^j r^m.
The closed-form AMOEBA numerator is (-1)^j (2j-1)!! + e^{-u} Q_j(u) with
Q_1 = 1 and Q_{j+1} = 3u (Q_j' - Q_j) - (2j+1) Q_j; its coefficients are
emitted too.

FP32 kernels evaluate N_j below the closed form's range from one table of
expansions on unit intervals: the series itself on [0, 1) (centre 0) and
re-centred Taylor expansions on the intervals above it, where the series
loses digits to alternating terms and the closed form to cancellation:
    N_j(c + t) = sum_n b_n t^n,  b_n = sum_k a_k C(k, n) c^(k - n),  |t| <= 1/2
with the exact series coefficients a_k; centres THOLE_CENTRES in x = a r,
AMOEBA_CENTRES in u = (a r)^3.  One table for the whole range keeps the
lanes of a warp on one code path whichever interval each lane's pair is in.

Run:  python gen_tables.py > series_tables.h
"""
from fractions import Fraction
from math import factorial

JMAX = 8      # highest radial derivative (tensor order) of the damped kernels
KT = 24       # Thole series length (powers of x)
KA = 30       # AMOEBA series length (powers of u)
NTAY = 16     # terms of each interval's expansion (a multiple of 4: rows are read as float4)
THOLE_CENTRES = (Fraction(0), Fraction(3, 2), Fraction(5, 2))
AMOEBA_CENTRES = (Fraction(0), Fraction(3, 2), Fraction(5, 2), Fraction(7, 2))
KFULL = 160   # series terms summed exactly for the re-centred coefficients


def power_rule(m, j):
    p = 1
    for i in range(j):
        p *= (m - 2 * i)
    return p


def thole(j, k):
    if k == 0:
        return Fraction(0)
    ck = Fraction((-1) ** (k + 1)) * (1 - Fraction(k, 2)) / factorial(k)
    return ck * power_rule(k - 1, j)


def amoeba(j, k):
    if j == 0 or k == 0:
        return Fraction(0)
    sk = Fraction((-1) ** k, factorial(k))
    return sk * power_rule(3 * k - 3, j - 1)


def amoeba_q():
    Q = [[Fraction(0)]]  # Q_0 unused
    q = [Fraction(1)]
    Q.append(q)
    for j in range(1, JMAX):
        n = [Fraction(0)] * (len(q) + 1)
        for d, c in enumerate(q):
            n[d] -= (2 * j + 1) * c
            n[d + 1] -= 3 * c
            if d >= 1:
                n[d] += 3 * d * c
        q = n
        Q.append(q)
    return Q


def binom(k, n):
    return factorial(k) // (factorial(n) * factorial(k - n))


def recentred(fn, j, c):
    """b_n, n < NTAY, of N_j(c + t) from the exact series fn(j, k)."""
    a = [fn(j, k) for k in range(KFULL)]
    return [sum(a[k] * binom(k, n) * c ** (k - n) for k in range(n, KFULL)) for n in range(NTAY)]


def fmt(fr):
    return repr(float(fr)) if fr != 0 else "0.0"


def main():
    out = []
    out.append("// Generated by gen_tables.py -- exact Taylor coefficients of the damped")
    out.append("// radial-derivative numerators (see that script for the definitions).")
    out.append("#pragma once")
    out.append(f"#define FMM_SER_JMAX {JMAX}")
    out.append(f"#define FMM_SER_KT {KT}")
    out.append(f"#define FMM_SER_KA {KA}")
    out.append("#define FMM_THOLE_SERIES_INIT { \\")
    for j in range(JMAX + 1):
        out.append("  {" + ", ".join(fmt(thole(j, k)) for k in range(KT + 1)) + "}, \\")
    out.append("}")
    out.append("#define FMM_AMOEBA_SERIES_INIT { \\")
    for j in range(JMAX + 1):
        out.append("  {" + ", ".join(fmt(amoeba(j, k)) for k in range(KA + 1)) + "}, \\")
    out.append("}")
    Q = amoeba_q()
    out.append("#define FMM_AMOEBA_Q_INIT { \\")
    for j in range(JMAX + 1):
        row = [Fraction(0)] * JMAX
        if j >= 1:
            for d, c in enumerate(Q[j]):
                row[d] = c
        out.append("  {" + ", ".join(fmt(c) for c in row) + "}, \\")
    out.append("}")
    out.append(f"#define FMM_TAY_N {NTAY}")
    out.append(f"#define FMM_THOLE_NC {len(THOLE_CENTRES)}")
    out.append(f"#define FMM_AMOEBA_NC {len(AMOEBA_CENTRES)}")
    for name, fn, cs in (("THOLE", thole, THOLE_CENTRES), ("AMOEBA", amoeba, AMOEBA_CENTRES)):
        out.append(f"#define FMM_{name}_TAY_INIT {{ \\")
        for j in range(JMAX + 1):
            rows = ["{" + ", ".join(fmt(b) for b in recentred(fn, j, c)) + "}" for c in cs]
            out.append("  {" + ", ".join(rows) + "}, \\")
        out.append("}")
    print("\n".join(out))


if __name__ == "__main__":
    main()

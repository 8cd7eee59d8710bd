#!/usr/bin/env python3
"""Generates oracle/harmonic_terms.h (test infrastructure): the field B = grad Phi
and its Jacobian of every harmonic-expansion term G(l, m), 0 <= l <= 5,
-l-1 <= m <= l+1, as expanded Cartesian polynomials.

Phi_lm = G * l! 2^|m| / (l+1+|m|)! * r^(l+1) P_(l+1)^|m|(cos theta)
         * (cos |m| phi for m >= 0, sin |m| phi for m < 0),
Legendre functions without the Condon-Shortley phase: the normalisation of
HarmonicExpandedBField (src/harmonicfields.cpp:50-829; e.g. G(0,0) is a
uniform Bz = G, G(1,-2) gives B = (G y, G x, 0)), derived here symbolically
from the definition so the oracle does not share the engine's Legendre
recursion.

    python3 oracle/gen_harmonic.py   (needs sympy)
"""
import os

import sympy as sp

x, y, z = sp.symbols("x y z", real=True)


def solid_harmonic(n, m):
    """r^n P_n^m(cos theta) e^{i m phi} in Cartesian form (no Condon-Shortley
    phase), from (x + i y)^m and the m-th derivative of P_n."""
    r2 = x * x + y * y + z * z
    t = sp.symbols("t")
    Pn = sp.legendre(n, t)
    dm = sp.diff(Pn, t, m)
    # r^n P_n^m(cos) = r^n sin^m d^m P_n(cos) -> (x+iy)^m * r^(n-m) dm(z/r)
    poly = sp.expand(dm.subs(t, z / sp.sqrt(r2)) * sp.sqrt(r2) ** (n - m))
    poly = sp.simplify(poly)
    return sp.expand(poly * (x + sp.I * y) ** m)


def phi(l, m):
    am = abs(m)
    c = sp.factorial(l) * 2 ** am / sp.factorial(l + 1 + am)
    h = solid_harmonic(l + 1, am)
    part = sp.re(h) if m >= 0 else sp.im(h)
    return sp.expand(c * part)


def main():
    lines = ["/* Generated by oracle/gen_harmonic.py from the definition of the",
             " * harmonic-expansion terms (test infrastructure; do not edit). */",
             "#pragma once",
             "#include <math.h>",
             "/* adds G times the (l, m) term's B (and dB[i][j] = dB_i/dx_j) at (x, y, z); false for unknown (l, m) */",
             "static inline bool harmonic_term(int l, int m, double G, double x, double y, double z, double B[3], double dB[3][3]) {"]
    for l in range(6):
        for m in range(-l - 1, l + 2):
            P = phi(l, m)
            Bc = [sp.expand(sp.diff(P, v)) for v in (x, y, z)]
            lines.append(f"    if (l == {l} && m == {m}) {{")
            for i, b in enumerate(Bc):
                lines.append(f"        B[{i}] += G * ({sp.ccode(b)});")
            lines.append("        if (dB) {")
            for i, b in enumerate(Bc):
                for j, v in enumerate((x, y, z)):
                    d = sp.expand(sp.diff(b, v))
                    if d != 0:
                        lines.append(f"            dB[{i}][{j}] += G * ({sp.ccode(d)});")
            lines.append("        }")
            lines.append("        return true;")
            lines.append("    }")
    lines.append("    (void)x; (void)y; (void)z;")
    lines.append("    return false;")
    lines.append("}")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "harmonic_terms.h")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()

"""Generate include/pt_constants.h: PENTrack's physical constants as exact double literals.

PENTrack defines its constants as ``long double`` (src/globals.cpp:13-32) and
derives the particle masses in eV/c^2 by a long-double division by the
elementary charge.  On x86-64 that is 80-bit extended arithmetic.  Device code
has no long double, and on aarch64 hosts ``long double`` is IEEE quad, so
the values are evaluated once here with numpy's x86 extended type, rounded
to double, and written as hex-float literals.  The oracle and the CUDA
kernels include the same header, so both see bit-identical constants.

Run on an x86-64 host:  python pentrack_gb300/csrc/gen_constants.py
"""
import os
import numpy as np

L = np.longdouble
assert np.finfo(L).nmant == 63, "needs x86 80-bit long double"

ele_e = L("1.602176487E-19")
c = {
    "PT_PI": L("3.1415926535897932384626"),
    "PT_ELE_E": ele_e,
    "PT_GRAVCONST": L("9.80665"),
    "PT_C0": L("299792458."),
    "PT_HBAR": L("1.05457266e-34"),
    "PT_M_N": L("1.674927211E-27") / ele_e,
    "PT_M_P": L("1.672621637E-27") / ele_e,
    "PT_M_E": L("9.10938215e-31") / ele_e,
    "PT_MU_N_SI": L("-0.96623641e-26"),
    "PT_GAMMA_N": L("-1.83247185e8"),
}
# species: (q [C], m [eV/c^2], mu [J/T], gamma [1/(T s)])  -- src/neutron.cpp:20, src/proton.cpp, src/electron.cpp
species = {
    "NEUTRON": (L(0), c["PT_M_N"], c["PT_MU_N_SI"], c["PT_GAMMA_N"]),
    "PROTON": (ele_e, c["PT_M_P"], L(0), L(0)),
    "ELECTRON": (-ele_e, c["PT_M_E"], L(0), L(0)),
}


def hx(v):
    return float(v).hex()


def main():
    out = os.path.join(os.path.dirname(__file__), "..", "..", "include", "pt_constants.h")
    lines = [
        "/* Generated by pentrack_gb300/csrc/gen_constants.py -- do not edit.",
        " * PENTrack's physical constants (src/globals.cpp:13-32), evaluated in x86",
        " * 80-bit long double as the reference does, then rounded once to double. */",
        "#ifndef PT_CONSTANTS_H",
        "#define PT_CONSTANTS_H",
        "",
    ]
    for k, v in c.items():
        lines.append(f"#define {k} {hx(v)} /* {float(v)!r} */")
    lines.append("")
    lines.append("/* Per-species derived constants: charge q [C], mass m [eV/c^2], magnetic moment mu [J/T],")
    lines.append(" * gyromagnetic ratio [1/(T s)], mass in kg (m*e), gravity force -g*m*e [N],")
    lines.append(" * mu/e [eV/T] and q/e, each computed in long double and rounded once. */")
    for name, (q, m, mu, g) in species.items():
        mkg = m * ele_e
        lines.append(f"#define PT_{name}_Q {hx(q)}")
        lines.append(f"#define PT_{name}_M {hx(m)}")
        lines.append(f"#define PT_{name}_MU {hx(mu)}")
        lines.append(f"#define PT_{name}_GAMMA {hx(g)}")
        lines.append(f"#define PT_{name}_MKG {hx(mkg)}")
        lines.append(f"#define PT_{name}_INV_MKG {hx(L(1) / mkg)}")
        lines.append(f"#define PT_{name}_FGRAV {hx(-c['PT_GRAVCONST'] * m * ele_e)}")
        lines.append(f"#define PT_{name}_MU_OVER_E {hx(mu / ele_e)}")
        lines.append(f"#define PT_{name}_Q_OVER_E {hx(q / ele_e)}")
        lines.append(f"#define PT_{name}_MC2 {hx(m * c['PT_C0'] * c['PT_C0'])}")
        lines.append(f"#define PT_{name}_MG {hx(m * c['PT_GRAVCONST'])}")
    lines.append("")
    lines.append("#define PT_C0_SQ " + hx(c["PT_C0"] * c["PT_C0"]))
    lines.append("#define PT_INV_C0_SQ " + hx(L(1) / (c["PT_C0"] * c["PT_C0"])))
    lines.append("#define PT_MAX_TRACK_DEVIATION 0x1.0624dd2f1a9fcp-10 /* 0.001 m, include/particle.h:20 */")
    lines.append("#define PT_REFLECT_TOLERANCE 1e-8 /* include/trianglemesh.h:39 */")
    lines.append("")
    lines.append("#endif")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", os.path.normpath(out))


if __name__ == "__main__":
    main()

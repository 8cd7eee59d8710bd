"""Generate the golden vectors under tests/golden from the reference's own code.

Run where the reference tree exists:  python tests/golden/gen_golden.py [REFERENCE_TREE]
(default: $PENTRACK_REFERENCE, else the build container's read-only mount).  It builds oracle/_ref/libptref.so (`make -C oracle ref`), i.e. the vendored
ALGLIB 3.15.0 and libtricubic sources of the reference compiled in place, and
records:
  alglib_spline.npz   spline1dgriddiffcubic(x, y) on uniform and random grids
                      (the call TabField3::CalcDerivs makes, src/field_3d.cpp:356)
  tricubic.npz        tricubic_get_coeff on random corner data
                      (TabField3::PreInterpol, src/field_3d.cpp:410) and
                      libtricubic's tricubic_eval value/derivatives at points
  reference_fixtures.npz  the IntegrationTest geometry/table and the unit-cube
                      STL read from the reference's test/ directory
  alglib_spline2d.npz spline2dbuildbicubicv + spline2ddiff / spline2dcalc on
                      uniform and random (r, z) grids (TabField, src/field_2d.cpp:247-335)
  alglib_spline1d.npz spline1dbuildcubic + spline1dcalc at random points and
                      the nodes (IntegrateSpin's axis spline, src/tracking.cpp:404-421)
  opera2d_tables.npz  test/VerticalLinearGradientField2D.tab and
                      test/CosineGradientField.tab read in centimetres
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    from pentrack_gb300.build import reference_tree
    tree = sys.argv[1] if len(sys.argv) > 1 else reference_tree()
    if not tree or not os.path.isdir(tree):
        sys.exit("reference tree not found: pass its path or set PENTRACK_REFERENCE")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref", f"REF={tree}"], check=True)
    from oracle import pyoracle
    from pentrack_gb300 import scenes

    R = pyoracle.ref_lib()
    assert R is not None
    dp = lambda a: a.ctypes.data_as(pyoracle.A.c_double_p)  # noqa: E731
    rng = np.random.default_rng(20191122)

    xs, ys, ds, ns = [], [], [], []
    for n in (2, 3, 4, 5, 7, 16, 64):
        for k in range(6):
            if k % 2 == 0:
                x = np.linspace(-0.21, 0.21, n)
            else:
                x = np.sort(rng.uniform(-1.0, 1.0, n))
                x[0] -= 0.5
            y = rng.normal(size=n) * (10.0 ** rng.integers(-6, 2))
            d = np.zeros(n)
            assert R.ref_spline_derivs(n, dp(x), dp(y), dp(d)) == 0
            xs.append(x); ys.append(y); ds.append(d); ns.append(n)
    off = np.cumsum([0] + ns)
    np.savez_compressed(os.path.join(HERE, "alglib_spline.npz"), n=np.array(ns), offset=off,
                        x=np.concatenate(xs), y=np.concatenate(ys), d=np.concatenate(ds))

    X = rng.normal(size=(64, 64))
    Acoef = np.zeros((64, 64))
    for i in range(64):
        R.ref_tricubic_coeff(dp(np.ascontiguousarray(X[i])), dp(Acoef[i]))
    pts = rng.uniform(0, 1, size=(64, 3))
    ev = np.zeros((64, 4))
    for i in range(64):
        a = np.ascontiguousarray(Acoef[i])
        for j, der in enumerate(((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1))):
            ev[i, j] = R.ref_tricubic_eval(dp(a), pts[i, 0], pts[i, 1], pts[i, 2], *der)
    np.savez_compressed(os.path.join(HERE, "tricubic.npz"), x=X, a=Acoef, pts=pts, eval=ev)

    ref = os.path.join(tree, "test")
    hollow = scenes.read_stl(os.path.join(ref, "HollowUnitCube.STL"))
    cube = scenes.read_stl(os.path.join(ref, "UnitCubeCenteredOn(0,0,0).STL"))
    axes, comps = scenes.read_opera3d(os.path.join(ref, "VerticalLinearGradientField3D.tab"), 0.01)
    np.savez_compressed(os.path.join(HERE, "reference_fixtures.npz"), hollow=hollow, cube=cube,
                        tab_x=axes[0], tab_y=axes[1], tab_z=axes[2], tab_bz=comps["BZ"], tab_bx=comps["BX"],
                        tab_by=comps["BY"], tab_v=comps["V"])
    cases = {}
    for case, (m, n) in enumerate(((2, 2), (3, 2), (2, 5), (4, 4), (7, 5), (11, 11), (6, 9))):
        if case % 2 == 0:
            x = np.linspace(0.0, 0.5, m)
            y = np.linspace(-0.2, 0.3, n)
        else:
            x = np.sort(rng.uniform(0.0, 1.0, m)) + 0.01 * np.arange(m)
            y = np.sort(rng.uniform(-1.0, 1.0, n)) + 0.01 * np.arange(n)
        F = rng.normal(size=(m, n)) * (10.0 ** rng.integers(-4, 3))  # [ix][iy]
        # TabField's range: x0 <= x < x0 + (x1 - x0)(m - 1), likewise in y (src/field_2d.cpp:291)
        xhi = min(x[-1], x[0] + (x[1] - x[0]) * (m - 1))
        yhi = min(y[-1], y[0] + (y[1] - y[0]) * (n - 1))
        px = np.concatenate([rng.uniform(x[0], xhi, 64), x[:-1], np.full(n - 1, x[0])])
        py = np.concatenate([rng.uniform(y[0], yhi, 64), np.full(m - 1, y[0]), y[:-1]])
        px, py = np.ascontiguousarray(px), np.ascontiguousarray(py)
        out = np.zeros((len(px), 5))
        fa = np.ascontiguousarray(F.T)  # ALGLIB's f[iy*m + ix]
        assert R.ref_spline2d(m, dp(x), n, dp(y), dp(fa), len(px), dp(px), dp(py), dp(out)) == 0
        cases.update({f"x{case}": x, f"y{case}": y, f"f{case}": F, f"px{case}": px, f"py{case}": py, f"out{case}": out})
    np.savez_compressed(os.path.join(HERE, "alglib_spline2d.npz"), n_cases=np.array(case + 1), **cases)

    sp1 = {}
    for case in range(8):
        n = (2, 3, 5, 11, 11, 11, 7, 11)[case]
        t0, t1 = rng.uniform(-1, 1), rng.uniform(1e-6, 2.0)
        x = np.array([t0 + i * (t1 - t0 + 1) / (n - 1) for i in range(n)])  # x1 + i (x2 - x1) / (n - 1), as IntegrateSpin
        y = rng.normal(size=n) * (10.0 ** rng.integers(-8, 3))
        pts = np.concatenate([rng.uniform(x[0] - 0.1 * (x[-1] - x[0]), x[-1] + 0.1 * (x[-1] - x[0]), 40), x])
        out = np.zeros(len(pts))
        assert R.ref_spline1d_calc(n, dp(x), dp(np.ascontiguousarray(y)), len(pts), dp(pts), dp(out)) == 0
        sp1.update({f"x{case}": x, f"y{case}": y, f"p{case}": pts, f"v{case}": out})
    np.savez_compressed(os.path.join(HERE, "alglib_spline1d.npz"), n_cases=np.array(8), **sp1)

    tabs = {}
    for key, name in (("linear", "VerticalLinearGradientField2D.tab"), ("cosine", "CosineGradientField.tab")):
        (r, z), cols = scenes.read_opera2d(os.path.join(ref, name), 0.01)
        tabs[f"{key}_r"], tabs[f"{key}_z"] = r, z
        for c, arr in cols.items():
            tabs[f"{key}_{c}"] = arr
    np.savez_compressed(os.path.join(HERE, "opera2d_tables.npz"), **tabs)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()

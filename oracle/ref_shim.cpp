/*
 * ref_shim.cpp -- C entry points over the reference's own vendored ALGLIB
 * 3.15.0 and libtricubic sources (TEST INFRASTRUCTURE).
 *
 * Built by `make -C oracle ref` into oracle/_ref/libptref.so, compiling the
 * sources where they lie in the reference tree.  Used only to pin the
 * oracle's restatements (spline derivatives of TabField3::CalcDerivs,
 * src/field_3d.cpp:336-364, and tricubic_get_coeff of TabField3::PreInterpol,
 * src/field_3d.cpp:367-414) and to generate tests/golden fixtures.
 */
#include "interpolation.h"
#include "tricubic.h"

extern "C" {

/* alglib::spline1dgriddiffcubic(x, y, d) exactly as TabField3::CalcDerivs calls it */
int ref_spline_derivs(int n, const double *x, const double *y, double *d) {
    try {
        alglib::real_1d_array xa, ya, da;
        xa.setcontent(n, x);
        ya.setcontent(n, y);
        da.setlength(n);
        alglib::spline1dgriddiffcubic(xa, ya, da);
        for (int i = 0; i < n; ++i) d[i] = da[i];
        return 0;
    } catch (...) {
        return -1;
    }
}

/* tricubic_get_coeff on the stacked layout [f, fx, fy, fz, fxy, fxz, fyz, fxyz] x 8 corners */
void ref_tricubic_coeff(const double *x64, double *a64) {
    double v[8][8];
    for (int d = 0; d < 8; ++d)
        for (int c = 0; c < 8; ++c) v[d][c] = x64[8 * d + c];
    tricubic_get_coeff(a64, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7]);
}

/* libtricubic's own evaluator (value and partial derivatives) */
double ref_tricubic_eval(double *a64, double x, double y, double z, int derx, int dery, int derz) {
    return tricubic_eval(a64, x, y, z, derx, dery, derz);
}
}

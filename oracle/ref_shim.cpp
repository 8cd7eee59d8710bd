/*
 * ref_shim.cpp -- C entry points over the reference's own vendored ALGLIB
 * 3.15.0 and libtricubic sources (TEST INFRASTRUCTURE).
 *
 * Built by `make -C oracle ref` into oracle/_ref/libptref.so, compiling the
 * sources where they lie in the reference tree.  Used only to pin the
 * oracle's restatements (spline derivatives of TabField3::CalcDerivs,
 * src/field_3d.cpp:336-364, tricubic_get_coeff of TabField3::PreInterpol,
 * src/field_3d.cpp:367-414, and the bicubic spline2d of TabField,
 * src/field_2d.cpp:232-399) and to generate tests/golden fixtures.
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

/* TabField's spline: spline2dbuildbicubicv(x, m, y, n, f, 1) on f[iy*m + ix]
 * (src/field_2d.cpp:247), then at each of np points spline2ddiff (out[5k..5k+3]
 * = f, df/dx, df/dy, d2f/dxdy) and spline2dcalc (out[5k+4]) */
int ref_spline2d(int m, const double *x, int n, const double *y, const double *f, int np, const double *px,
                 const double *py, double *out) {
    try {
        alglib::real_1d_array xa, ya, fa;
        xa.setcontent(m, x);
        ya.setcontent(n, y);
        fa.setcontent((alglib::ae_int_t)m * n, f);
        alglib::spline2dinterpolant c;
        alglib::spline2dbuildbicubicv(xa, m, ya, n, fa, 1, c);
        for (int k = 0; k < np; ++k) {
            double v, dx, dy, dxy;
            alglib::spline2ddiff(c, px[k], py[k], v, dx, dy, dxy);
            out[5 * k + 0] = v;
            out[5 * k + 1] = dx;
            out[5 * k + 2] = dy;
            out[5 * k + 3] = dxy;
            out[5 * k + 4] = alglib::spline2dcalc(c, px[k], py[k]);
        }
        return 0;
    } catch (...) {
        return -1;
    }
}

/* IntegrateSpin's axis spline: spline1dbuildcubic(x, y) (the short form,
 * src/tracking.cpp:419) and spline1dcalc at np points */
int ref_spline1d_calc(int n, const double *x, const double *y, int np, const double *pts, double *out) {
    try {
        alglib::real_1d_array xa, ya;
        xa.setcontent(n, x);
        ya.setcontent(n, y);
        alglib::spline1dinterpolant c;
        alglib::spline1dbuildcubic(xa, ya, c);
        for (int k = 0; k < np; ++k) out[k] = alglib::spline1dcalc(c, pts[k]);
        return 0;
    } catch (...) {
        return -1;
    }
}
}

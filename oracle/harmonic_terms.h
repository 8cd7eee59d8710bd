/* Generated by oracle/gen_harmonic.py from the definition of the
 * harmonic-expansion terms (test infrastructure; do not edit). */
#pragma once
#include <math.h>
/* adds G times the (l, m) term's B (and dB[i][j] = dB_i/dx_j) at (x, y, z); false for unknown (l, m) */
static inline bool harmonic_term(int l, int m, double G, double x, double y, double z, double B[3], double dB[3][3]) {
    if (l == 0 && m == -1) {
        B[0] += G * (0);
        B[1] += G * (1);
        B[2] += G * (0);
        if (dB) {
        }
        return true;
    }
    if (l == 0 && m == 0) {
        B[0] += G * (0);
        B[1] += G * (0);
        B[2] += G * (1);
        if (dB) {
        }
        return true;
    }
    if (l == 0 && m == 1) {
        B[0] += G * (1);
        B[1] += G * (0);
        B[2] += G * (0);
        if (dB) {
        }
        return true;
    }
    if (l == 1 && m == -2) {
        B[0] += G * (y);
        B[1] += G * (x);
        B[2] += G * (0);
        if (dB) {
            dB[0][1] += G * (1);
            dB[1][0] += G * (1);
        }
        return true;
    }
    if (l == 1 && m == -1) {
        B[0] += G * (0);
        B[1] += G * (z);
        B[2] += G * (y);
        if (dB) {
            dB[1][2] += G * (1);
            dB[2][1] += G * (1);
        }
        return true;
    }
    if (l == 1 && m == 0) {
        B[0] += G * (-1.0/2.0*x);
        B[1] += G * (-1.0/2.0*y);
        B[2] += G * (z);
        if (dB) {
            dB[0][0] += G * (-1.0/2.0);
            dB[1][1] += G * (-1.0/2.0);
            dB[2][2] += G * (1);
        }
        return true;
    }
    if (l == 1 && m == 1) {
        B[0] += G * (z);
        B[1] += G * (0);
        B[2] += G * (x);
        if (dB) {
            dB[0][2] += G * (1);
            dB[2][0] += G * (1);
        }
        return true;
    }
    if (l == 1 && m == 2) {
        B[0] += G * (x);
        B[1] += G * (-y);
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (1);
            dB[1][1] += G * (-1);
        }
        return true;
    }
    if (l == 2 && m == -3) {
        B[0] += G * (2*x*y);
        B[1] += G * (pow(x, 2) - pow(y, 2));
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (2*y);
            dB[0][1] += G * (2*x);
            dB[1][0] += G * (2*x);
            dB[1][1] += G * (-2*y);
        }
        return true;
    }
    if (l == 2 && m == -2) {
        B[0] += G * (2*y*z);
        B[1] += G * (2*x*z);
        B[2] += G * (2*x*y);
        if (dB) {
            dB[0][1] += G * (2*z);
            dB[0][2] += G * (2*y);
            dB[1][0] += G * (2*z);
            dB[1][2] += G * (2*x);
            dB[2][0] += G * (2*y);
            dB[2][1] += G * (2*x);
        }
        return true;
    }
    if (l == 2 && m == -1) {
        B[0] += G * (-1.0/2.0*x*y);
        B[1] += G * (-1.0/4.0*pow(x, 2) - 3.0/4.0*pow(y, 2) + pow(z, 2));
        B[2] += G * (2*y*z);
        if (dB) {
            dB[0][0] += G * (-1.0/2.0*y);
            dB[0][1] += G * (-1.0/2.0*x);
            dB[1][0] += G * (-1.0/2.0*x);
            dB[1][1] += G * (-3.0/2.0*y);
            dB[1][2] += G * (2*z);
            dB[2][1] += G * (2*z);
            dB[2][2] += G * (2*y);
        }
        return true;
    }
    if (l == 2 && m == 0) {
        B[0] += G * (-x*z);
        B[1] += G * (-y*z);
        B[2] += G * (-1.0/2.0*pow(x, 2) - 1.0/2.0*pow(y, 2) + pow(z, 2));
        if (dB) {
            dB[0][0] += G * (-z);
            dB[0][2] += G * (-x);
            dB[1][1] += G * (-z);
            dB[1][2] += G * (-y);
            dB[2][0] += G * (-x);
            dB[2][1] += G * (-y);
            dB[2][2] += G * (2*z);
        }
        return true;
    }
    if (l == 2 && m == 1) {
        B[0] += G * (-3.0/4.0*pow(x, 2) - 1.0/4.0*pow(y, 2) + pow(z, 2));
        B[1] += G * (-1.0/2.0*x*y);
        B[2] += G * (2*x*z);
        if (dB) {
            dB[0][0] += G * (-3.0/2.0*x);
            dB[0][1] += G * (-1.0/2.0*y);
            dB[0][2] += G * (2*z);
            dB[1][0] += G * (-1.0/2.0*y);
            dB[1][1] += G * (-1.0/2.0*x);
            dB[2][0] += G * (2*z);
            dB[2][2] += G * (2*x);
        }
        return true;
    }
    if (l == 2 && m == 2) {
        B[0] += G * (2*x*z);
        B[1] += G * (-2*y*z);
        B[2] += G * (pow(x, 2) - pow(y, 2));
        if (dB) {
            dB[0][0] += G * (2*z);
            dB[0][2] += G * (2*x);
            dB[1][1] += G * (-2*z);
            dB[1][2] += G * (-2*y);
            dB[2][0] += G * (2*x);
            dB[2][1] += G * (-2*y);
        }
        return true;
    }
    if (l == 2 && m == 3) {
        B[0] += G * (pow(x, 2) - pow(y, 2));
        B[1] += G * (-2*x*y);
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (2*x);
            dB[0][1] += G * (-2*y);
            dB[1][0] += G * (-2*y);
            dB[1][1] += G * (-2*x);
        }
        return true;
    }
    if (l == 3 && m == -4) {
        B[0] += G * (3*pow(x, 2)*y - pow(y, 3));
        B[1] += G * (pow(x, 3) - 3*x*pow(y, 2));
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (6*x*y);
            dB[0][1] += G * (3*pow(x, 2) - 3*pow(y, 2));
            dB[1][0] += G * (3*pow(x, 2) - 3*pow(y, 2));
            dB[1][1] += G * (-6*x*y);
        }
        return true;
    }
    if (l == 3 && m == -3) {
        B[0] += G * (6*x*y*z);
        B[1] += G * (3*pow(x, 2)*z - 3*pow(y, 2)*z);
        B[2] += G * (3*pow(x, 2)*y - pow(y, 3));
        if (dB) {
            dB[0][0] += G * (6*y*z);
            dB[0][1] += G * (6*x*z);
            dB[0][2] += G * (6*x*y);
            dB[1][0] += G * (6*x*z);
            dB[1][1] += G * (-6*y*z);
            dB[1][2] += G * (3*pow(x, 2) - 3*pow(y, 2));
            dB[2][0] += G * (6*x*y);
            dB[2][1] += G * (3*pow(x, 2) - 3*pow(y, 2));
        }
        return true;
    }
    if (l == 3 && m == -2) {
        B[0] += G * (-3.0/2.0*pow(x, 2)*y - 1.0/2.0*pow(y, 3) + 3*y*pow(z, 2));
        B[1] += G * (-1.0/2.0*pow(x, 3) - 3.0/2.0*x*pow(y, 2) + 3*x*pow(z, 2));
        B[2] += G * (6*x*y*z);
        if (dB) {
            dB[0][0] += G * (-3*x*y);
            dB[0][1] += G * (-3.0/2.0*pow(x, 2) - 3.0/2.0*pow(y, 2) + 3*pow(z, 2));
            dB[0][2] += G * (6*y*z);
            dB[1][0] += G * (-3.0/2.0*pow(x, 2) - 3.0/2.0*pow(y, 2) + 3*pow(z, 2));
            dB[1][1] += G * (-3*x*y);
            dB[1][2] += G * (6*x*z);
            dB[2][0] += G * (6*y*z);
            dB[2][1] += G * (6*x*z);
            dB[2][2] += G * (6*x*y);
        }
        return true;
    }
    if (l == 3 && m == -1) {
        B[0] += G * (-3.0/2.0*x*y*z);
        B[1] += G * (-3.0/4.0*pow(x, 2)*z - 9.0/4.0*pow(y, 2)*z + pow(z, 3));
        B[2] += G * (-3.0/4.0*pow(x, 2)*y - 3.0/4.0*pow(y, 3) + 3*y*pow(z, 2));
        if (dB) {
            dB[0][0] += G * (-3.0/2.0*y*z);
            dB[0][1] += G * (-3.0/2.0*x*z);
            dB[0][2] += G * (-3.0/2.0*x*y);
            dB[1][0] += G * (-3.0/2.0*x*z);
            dB[1][1] += G * (-9.0/2.0*y*z);
            dB[1][2] += G * (-3.0/4.0*pow(x, 2) - 9.0/4.0*pow(y, 2) + 3*pow(z, 2));
            dB[2][0] += G * (-3.0/2.0*x*y);
            dB[2][1] += G * (-3.0/4.0*pow(x, 2) - 9.0/4.0*pow(y, 2) + 3*pow(z, 2));
            dB[2][2] += G * (6*y*z);
        }
        return true;
    }
    if (l == 3 && m == 0) {
        B[0] += G * ((3.0/8.0)*pow(x, 3) + (3.0/8.0)*x*pow(y, 2) - 3.0/2.0*x*pow(z, 2));
        B[1] += G * ((3.0/8.0)*pow(x, 2)*y + (3.0/8.0)*pow(y, 3) - 3.0/2.0*y*pow(z, 2));
        B[2] += G * (-3.0/2.0*pow(x, 2)*z - 3.0/2.0*pow(y, 2)*z + pow(z, 3));
        if (dB) {
            dB[0][0] += G * ((9.0/8.0)*pow(x, 2) + (3.0/8.0)*pow(y, 2) - 3.0/2.0*pow(z, 2));
            dB[0][1] += G * ((3.0/4.0)*x*y);
            dB[0][2] += G * (-3*x*z);
            dB[1][0] += G * ((3.0/4.0)*x*y);
            dB[1][1] += G * ((3.0/8.0)*pow(x, 2) + (9.0/8.0)*pow(y, 2) - 3.0/2.0*pow(z, 2));
            dB[1][2] += G * (-3*y*z);
            dB[2][0] += G * (-3*x*z);
            dB[2][1] += G * (-3*y*z);
            dB[2][2] += G * (-3.0/2.0*pow(x, 2) - 3.0/2.0*pow(y, 2) + 3*pow(z, 2));
        }
        return true;
    }
    if (l == 3 && m == 1) {
        B[0] += G * (-9.0/4.0*pow(x, 2)*z - 3.0/4.0*pow(y, 2)*z + pow(z, 3));
        B[1] += G * (-3.0/2.0*x*y*z);
        B[2] += G * (-3.0/4.0*pow(x, 3) - 3.0/4.0*x*pow(y, 2) + 3*x*pow(z, 2));
        if (dB) {
            dB[0][0] += G * (-9.0/2.0*x*z);
            dB[0][1] += G * (-3.0/2.0*y*z);
            dB[0][2] += G * (-9.0/4.0*pow(x, 2) - 3.0/4.0*pow(y, 2) + 3*pow(z, 2));
            dB[1][0] += G * (-3.0/2.0*y*z);
            dB[1][1] += G * (-3.0/2.0*x*z);
            dB[1][2] += G * (-3.0/2.0*x*y);
            dB[2][0] += G * (-9.0/4.0*pow(x, 2) - 3.0/4.0*pow(y, 2) + 3*pow(z, 2));
            dB[2][1] += G * (-3.0/2.0*x*y);
            dB[2][2] += G * (6*x*z);
        }
        return true;
    }
    if (l == 3 && m == 2) {
        B[0] += G * (-pow(x, 3) + 3*x*pow(z, 2));
        B[1] += G * (pow(y, 3) - 3*y*pow(z, 2));
        B[2] += G * (3*pow(x, 2)*z - 3*pow(y, 2)*z);
        if (dB) {
            dB[0][0] += G * (-3*pow(x, 2) + 3*pow(z, 2));
            dB[0][2] += G * (6*x*z);
            dB[1][1] += G * (3*pow(y, 2) - 3*pow(z, 2));
            dB[1][2] += G * (-6*y*z);
            dB[2][0] += G * (6*x*z);
            dB[2][1] += G * (-6*y*z);
            dB[2][2] += G * (3*pow(x, 2) - 3*pow(y, 2));
        }
        return true;
    }
    if (l == 3 && m == 3) {
        B[0] += G * (3*pow(x, 2)*z - 3*pow(y, 2)*z);
        B[1] += G * (-6*x*y*z);
        B[2] += G * (pow(x, 3) - 3*x*pow(y, 2));
        if (dB) {
            dB[0][0] += G * (6*x*z);
            dB[0][1] += G * (-6*y*z);
            dB[0][2] += G * (3*pow(x, 2) - 3*pow(y, 2));
            dB[1][0] += G * (-6*y*z);
            dB[1][1] += G * (-6*x*z);
            dB[1][2] += G * (-6*x*y);
            dB[2][0] += G * (3*pow(x, 2) - 3*pow(y, 2));
            dB[2][1] += G * (-6*x*y);
        }
        return true;
    }
    if (l == 3 && m == 4) {
        B[0] += G * (pow(x, 3) - 3*x*pow(y, 2));
        B[1] += G * (-3*pow(x, 2)*y + pow(y, 3));
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (3*pow(x, 2) - 3*pow(y, 2));
            dB[0][1] += G * (-6*x*y);
            dB[1][0] += G * (-6*x*y);
            dB[1][1] += G * (-3*pow(x, 2) + 3*pow(y, 2));
        }
        return true;
    }
    if (l == 4 && m == -5) {
        B[0] += G * (4*pow(x, 3)*y - 4*x*pow(y, 3));
        B[1] += G * (pow(x, 4) - 6*pow(x, 2)*pow(y, 2) + pow(y, 4));
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (12*pow(x, 2)*y - 4*pow(y, 3));
            dB[0][1] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
            dB[1][0] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
            dB[1][1] += G * (-12*pow(x, 2)*y + 4*pow(y, 3));
        }
        return true;
    }
    if (l == 4 && m == -4) {
        B[0] += G * (12*pow(x, 2)*y*z - 4*pow(y, 3)*z);
        B[1] += G * (4*pow(x, 3)*z - 12*x*pow(y, 2)*z);
        B[2] += G * (4*pow(x, 3)*y - 4*x*pow(y, 3));
        if (dB) {
            dB[0][0] += G * (24*x*y*z);
            dB[0][1] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
            dB[0][2] += G * (12*pow(x, 2)*y - 4*pow(y, 3));
            dB[1][0] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
            dB[1][1] += G * (-24*x*y*z);
            dB[1][2] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
            dB[2][0] += G * (12*pow(x, 2)*y - 4*pow(y, 3));
            dB[2][1] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
        }
        return true;
    }
    if (l == 4 && m == -3) {
        B[0] += G * (-3*pow(x, 3)*y - x*pow(y, 3) + 12*x*y*pow(z, 2));
        B[1] += G * (-3.0/4.0*pow(x, 4) - 3.0/2.0*pow(x, 2)*pow(y, 2) + 6*pow(x, 2)*pow(z, 2) + (5.0/4.0)*pow(y, 4) - 6*pow(y, 2)*pow(z, 2));
        B[2] += G * (12*pow(x, 2)*y*z - 4*pow(y, 3)*z);
        if (dB) {
            dB[0][0] += G * (-9*pow(x, 2)*y - pow(y, 3) + 12*y*pow(z, 2));
            dB[0][1] += G * (-3*pow(x, 3) - 3*x*pow(y, 2) + 12*x*pow(z, 2));
            dB[0][2] += G * (24*x*y*z);
            dB[1][0] += G * (-3*pow(x, 3) - 3*x*pow(y, 2) + 12*x*pow(z, 2));
            dB[1][1] += G * (-3*pow(x, 2)*y + 5*pow(y, 3) - 12*y*pow(z, 2));
            dB[1][2] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
            dB[2][0] += G * (24*x*y*z);
            dB[2][1] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
            dB[2][2] += G * (12*pow(x, 2)*y - 4*pow(y, 3));
        }
        return true;
    }
    if (l == 4 && m == -2) {
        B[0] += G * (-6*pow(x, 2)*y*z - 2*pow(y, 3)*z + 4*y*pow(z, 3));
        B[1] += G * (-2*pow(x, 3)*z - 6*x*pow(y, 2)*z + 4*x*pow(z, 3));
        B[2] += G * (-2*pow(x, 3)*y - 2*x*pow(y, 3) + 12*x*y*pow(z, 2));
        if (dB) {
            dB[0][0] += G * (-12*x*y*z);
            dB[0][1] += G * (-6*pow(x, 2)*z - 6*pow(y, 2)*z + 4*pow(z, 3));
            dB[0][2] += G * (-6*pow(x, 2)*y - 2*pow(y, 3) + 12*y*pow(z, 2));
            dB[1][0] += G * (-6*pow(x, 2)*z - 6*pow(y, 2)*z + 4*pow(z, 3));
            dB[1][1] += G * (-12*x*y*z);
            dB[1][2] += G * (-2*pow(x, 3) - 6*x*pow(y, 2) + 12*x*pow(z, 2));
            dB[2][0] += G * (-6*pow(x, 2)*y - 2*pow(y, 3) + 12*y*pow(z, 2));
            dB[2][1] += G * (-2*pow(x, 3) - 6*x*pow(y, 2) + 12*x*pow(z, 2));
            dB[2][2] += G * (24*x*y*z);
        }
        return true;
    }
    if (l == 4 && m == -1) {
        B[0] += G * ((1.0/2.0)*pow(x, 3)*y + (1.0/2.0)*x*pow(y, 3) - 3*x*y*pow(z, 2));
        B[1] += G * ((1.0/8.0)*pow(x, 4) + (3.0/4.0)*pow(x, 2)*pow(y, 2) - 3.0/2.0*pow(x, 2)*pow(z, 2) + (5.0/8.0)*pow(y, 4) - 9.0/2.0*pow(y, 2)*pow(z, 2) + pow(z, 4));
        B[2] += G * (-3*pow(x, 2)*y*z - 3*pow(y, 3)*z + 4*y*pow(z, 3));
        if (dB) {
            dB[0][0] += G * ((3.0/2.0)*pow(x, 2)*y + (1.0/2.0)*pow(y, 3) - 3*y*pow(z, 2));
            dB[0][1] += G * ((1.0/2.0)*pow(x, 3) + (3.0/2.0)*x*pow(y, 2) - 3*x*pow(z, 2));
            dB[0][2] += G * (-6*x*y*z);
            dB[1][0] += G * ((1.0/2.0)*pow(x, 3) + (3.0/2.0)*x*pow(y, 2) - 3*x*pow(z, 2));
            dB[1][1] += G * ((3.0/2.0)*pow(x, 2)*y + (5.0/2.0)*pow(y, 3) - 9*y*pow(z, 2));
            dB[1][2] += G * (-3*pow(x, 2)*z - 9*pow(y, 2)*z + 4*pow(z, 3));
            dB[2][0] += G * (-6*x*y*z);
            dB[2][1] += G * (-3*pow(x, 2)*z - 9*pow(y, 2)*z + 4*pow(z, 3));
            dB[2][2] += G * (-3*pow(x, 2)*y - 3*pow(y, 3) + 12*y*pow(z, 2));
        }
        return true;
    }
    if (l == 4 && m == 0) {
        B[0] += G * ((3.0/2.0)*pow(x, 3)*z + (3.0/2.0)*x*pow(y, 2)*z - 2*x*pow(z, 3));
        B[1] += G * ((3.0/2.0)*pow(x, 2)*y*z + (3.0/2.0)*pow(y, 3)*z - 2*y*pow(z, 3));
        B[2] += G * ((3.0/8.0)*pow(x, 4) + (3.0/4.0)*pow(x, 2)*pow(y, 2) - 3*pow(x, 2)*pow(z, 2) + (3.0/8.0)*pow(y, 4) - 3*pow(y, 2)*pow(z, 2) + pow(z, 4));
        if (dB) {
            dB[0][0] += G * ((9.0/2.0)*pow(x, 2)*z + (3.0/2.0)*pow(y, 2)*z - 2*pow(z, 3));
            dB[0][1] += G * (3*x*y*z);
            dB[0][2] += G * ((3.0/2.0)*pow(x, 3) + (3.0/2.0)*x*pow(y, 2) - 6*x*pow(z, 2));
            dB[1][0] += G * (3*x*y*z);
            dB[1][1] += G * ((3.0/2.0)*pow(x, 2)*z + (9.0/2.0)*pow(y, 2)*z - 2*pow(z, 3));
            dB[1][2] += G * ((3.0/2.0)*pow(x, 2)*y + (3.0/2.0)*pow(y, 3) - 6*y*pow(z, 2));
            dB[2][0] += G * ((3.0/2.0)*pow(x, 3) + (3.0/2.0)*x*pow(y, 2) - 6*x*pow(z, 2));
            dB[2][1] += G * ((3.0/2.0)*pow(x, 2)*y + (3.0/2.0)*pow(y, 3) - 6*y*pow(z, 2));
            dB[2][2] += G * (-6*pow(x, 2)*z - 6*pow(y, 2)*z + 4*pow(z, 3));
        }
        return true;
    }
    if (l == 4 && m == 1) {
        B[0] += G * ((5.0/8.0)*pow(x, 4) + (3.0/4.0)*pow(x, 2)*pow(y, 2) - 9.0/2.0*pow(x, 2)*pow(z, 2) + (1.0/8.0)*pow(y, 4) - 3.0/2.0*pow(y, 2)*pow(z, 2) + pow(z, 4));
        B[1] += G * ((1.0/2.0)*pow(x, 3)*y + (1.0/2.0)*x*pow(y, 3) - 3*x*y*pow(z, 2));
        B[2] += G * (-3*pow(x, 3)*z - 3*x*pow(y, 2)*z + 4*x*pow(z, 3));
        if (dB) {
            dB[0][0] += G * ((5.0/2.0)*pow(x, 3) + (3.0/2.0)*x*pow(y, 2) - 9*x*pow(z, 2));
            dB[0][1] += G * ((3.0/2.0)*pow(x, 2)*y + (1.0/2.0)*pow(y, 3) - 3*y*pow(z, 2));
            dB[0][2] += G * (-9*pow(x, 2)*z - 3*pow(y, 2)*z + 4*pow(z, 3));
            dB[1][0] += G * ((3.0/2.0)*pow(x, 2)*y + (1.0/2.0)*pow(y, 3) - 3*y*pow(z, 2));
            dB[1][1] += G * ((1.0/2.0)*pow(x, 3) + (3.0/2.0)*x*pow(y, 2) - 3*x*pow(z, 2));
            dB[1][2] += G * (-6*x*y*z);
            dB[2][0] += G * (-9*pow(x, 2)*z - 3*pow(y, 2)*z + 4*pow(z, 3));
            dB[2][1] += G * (-6*x*y*z);
            dB[2][2] += G * (-3*pow(x, 3) - 3*x*pow(y, 2) + 12*x*pow(z, 2));
        }
        return true;
    }
    if (l == 4 && m == 2) {
        B[0] += G * (-4*pow(x, 3)*z + 4*x*pow(z, 3));
        B[1] += G * (4*pow(y, 3)*z - 4*y*pow(z, 3));
        B[2] += G * (-pow(x, 4) + 6*pow(x, 2)*pow(z, 2) + pow(y, 4) - 6*pow(y, 2)*pow(z, 2));
        if (dB) {
            dB[0][0] += G * (-12*pow(x, 2)*z + 4*pow(z, 3));
            dB[0][2] += G * (-4*pow(x, 3) + 12*x*pow(z, 2));
            dB[1][1] += G * (12*pow(y, 2)*z - 4*pow(z, 3));
            dB[1][2] += G * (4*pow(y, 3) - 12*y*pow(z, 2));
            dB[2][0] += G * (-4*pow(x, 3) + 12*x*pow(z, 2));
            dB[2][1] += G * (4*pow(y, 3) - 12*y*pow(z, 2));
            dB[2][2] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
        }
        return true;
    }
    if (l == 4 && m == 3) {
        B[0] += G * (-5.0/4.0*pow(x, 4) + (3.0/2.0)*pow(x, 2)*pow(y, 2) + 6*pow(x, 2)*pow(z, 2) + (3.0/4.0)*pow(y, 4) - 6*pow(y, 2)*pow(z, 2));
        B[1] += G * (pow(x, 3)*y + 3*x*pow(y, 3) - 12*x*y*pow(z, 2));
        B[2] += G * (4*pow(x, 3)*z - 12*x*pow(y, 2)*z);
        if (dB) {
            dB[0][0] += G * (-5*pow(x, 3) + 3*x*pow(y, 2) + 12*x*pow(z, 2));
            dB[0][1] += G * (3*pow(x, 2)*y + 3*pow(y, 3) - 12*y*pow(z, 2));
            dB[0][2] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
            dB[1][0] += G * (3*pow(x, 2)*y + 3*pow(y, 3) - 12*y*pow(z, 2));
            dB[1][1] += G * (pow(x, 3) + 9*x*pow(y, 2) - 12*x*pow(z, 2));
            dB[1][2] += G * (-24*x*y*z);
            dB[2][0] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
            dB[2][1] += G * (-24*x*y*z);
            dB[2][2] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
        }
        return true;
    }
    if (l == 4 && m == 4) {
        B[0] += G * (4*pow(x, 3)*z - 12*x*pow(y, 2)*z);
        B[1] += G * (-12*pow(x, 2)*y*z + 4*pow(y, 3)*z);
        B[2] += G * (pow(x, 4) - 6*pow(x, 2)*pow(y, 2) + pow(y, 4));
        if (dB) {
            dB[0][0] += G * (12*pow(x, 2)*z - 12*pow(y, 2)*z);
            dB[0][1] += G * (-24*x*y*z);
            dB[0][2] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
            dB[1][0] += G * (-24*x*y*z);
            dB[1][1] += G * (-12*pow(x, 2)*z + 12*pow(y, 2)*z);
            dB[1][2] += G * (-12*pow(x, 2)*y + 4*pow(y, 3));
            dB[2][0] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
            dB[2][1] += G * (-12*pow(x, 2)*y + 4*pow(y, 3));
        }
        return true;
    }
    if (l == 4 && m == 5) {
        B[0] += G * (pow(x, 4) - 6*pow(x, 2)*pow(y, 2) + pow(y, 4));
        B[1] += G * (-4*pow(x, 3)*y + 4*x*pow(y, 3));
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (4*pow(x, 3) - 12*x*pow(y, 2));
            dB[0][1] += G * (-12*pow(x, 2)*y + 4*pow(y, 3));
            dB[1][0] += G * (-12*pow(x, 2)*y + 4*pow(y, 3));
            dB[1][1] += G * (-4*pow(x, 3) + 12*x*pow(y, 2));
        }
        return true;
    }
    if (l == 5 && m == -6) {
        B[0] += G * (5*pow(x, 4)*y - 10*pow(x, 2)*pow(y, 3) + pow(y, 5));
        B[1] += G * (pow(x, 5) - 10*pow(x, 3)*pow(y, 2) + 5*x*pow(y, 4));
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (20*pow(x, 3)*y - 20*x*pow(y, 3));
            dB[0][1] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
            dB[1][0] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
            dB[1][1] += G * (-20*pow(x, 3)*y + 20*x*pow(y, 3));
        }
        return true;
    }
    if (l == 5 && m == -5) {
        B[0] += G * (20*pow(x, 3)*y*z - 20*x*pow(y, 3)*z);
        B[1] += G * (5*pow(x, 4)*z - 30*pow(x, 2)*pow(y, 2)*z + 5*pow(y, 4)*z);
        B[2] += G * (5*pow(x, 4)*y - 10*pow(x, 2)*pow(y, 3) + pow(y, 5));
        if (dB) {
            dB[0][0] += G * (60*pow(x, 2)*y*z - 20*pow(y, 3)*z);
            dB[0][1] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
            dB[0][2] += G * (20*pow(x, 3)*y - 20*x*pow(y, 3));
            dB[1][0] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
            dB[1][1] += G * (-60*pow(x, 2)*y*z + 20*pow(y, 3)*z);
            dB[1][2] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
            dB[2][0] += G * (20*pow(x, 3)*y - 20*x*pow(y, 3));
            dB[2][1] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
        }
        return true;
    }
    if (l == 5 && m == -4) {
        B[0] += G * (-5*pow(x, 4)*y + 30*pow(x, 2)*y*pow(z, 2) + pow(y, 5) - 10*pow(y, 3)*pow(z, 2));
        B[1] += G * (-pow(x, 5) + 10*pow(x, 3)*pow(z, 2) + 5*x*pow(y, 4) - 30*x*pow(y, 2)*pow(z, 2));
        B[2] += G * (20*pow(x, 3)*y*z - 20*x*pow(y, 3)*z);
        if (dB) {
            dB[0][0] += G * (-20*pow(x, 3)*y + 60*x*y*pow(z, 2));
            dB[0][1] += G * (-5*pow(x, 4) + 30*pow(x, 2)*pow(z, 2) + 5*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
            dB[0][2] += G * (60*pow(x, 2)*y*z - 20*pow(y, 3)*z);
            dB[1][0] += G * (-5*pow(x, 4) + 30*pow(x, 2)*pow(z, 2) + 5*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
            dB[1][1] += G * (20*x*pow(y, 3) - 60*x*y*pow(z, 2));
            dB[1][2] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
            dB[2][0] += G * (60*pow(x, 2)*y*z - 20*pow(y, 3)*z);
            dB[2][1] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
            dB[2][2] += G * (20*pow(x, 3)*y - 20*x*pow(y, 3));
        }
        return true;
    }
    if (l == 5 && m == -3) {
        B[0] += G * (-15*pow(x, 3)*y*z - 5*x*pow(y, 3)*z + 20*x*y*pow(z, 3));
        B[1] += G * (-15.0/4.0*pow(x, 4)*z - 15.0/2.0*pow(x, 2)*pow(y, 2)*z + 10*pow(x, 2)*pow(z, 3) + (25.0/4.0)*pow(y, 4)*z - 10*pow(y, 2)*pow(z, 3));
        B[2] += G * (-15.0/4.0*pow(x, 4)*y - 5.0/2.0*pow(x, 2)*pow(y, 3) + 30*pow(x, 2)*y*pow(z, 2) + (5.0/4.0)*pow(y, 5) - 10*pow(y, 3)*pow(z, 2));
        if (dB) {
            dB[0][0] += G * (-45*pow(x, 2)*y*z - 5*pow(y, 3)*z + 20*y*pow(z, 3));
            dB[0][1] += G * (-15*pow(x, 3)*z - 15*x*pow(y, 2)*z + 20*x*pow(z, 3));
            dB[0][2] += G * (-15*pow(x, 3)*y - 5*x*pow(y, 3) + 60*x*y*pow(z, 2));
            dB[1][0] += G * (-15*pow(x, 3)*z - 15*x*pow(y, 2)*z + 20*x*pow(z, 3));
            dB[1][1] += G * (-15*pow(x, 2)*y*z + 25*pow(y, 3)*z - 20*y*pow(z, 3));
            dB[1][2] += G * (-15.0/4.0*pow(x, 4) - 15.0/2.0*pow(x, 2)*pow(y, 2) + 30*pow(x, 2)*pow(z, 2) + (25.0/4.0)*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
            dB[2][0] += G * (-15*pow(x, 3)*y - 5*x*pow(y, 3) + 60*x*y*pow(z, 2));
            dB[2][1] += G * (-15.0/4.0*pow(x, 4) - 15.0/2.0*pow(x, 2)*pow(y, 2) + 30*pow(x, 2)*pow(z, 2) + (25.0/4.0)*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
            dB[2][2] += G * (60*pow(x, 2)*y*z - 20*pow(y, 3)*z);
        }
        return true;
    }
    if (l == 5 && m == -2) {
        B[0] += G * ((25.0/16.0)*pow(x, 4)*y + (15.0/8.0)*pow(x, 2)*pow(y, 3) - 15*pow(x, 2)*y*pow(z, 2) + (5.0/16.0)*pow(y, 5) - 5*pow(y, 3)*pow(z, 2) + 5*y*pow(z, 4));
        B[1] += G * ((5.0/16.0)*pow(x, 5) + (15.0/8.0)*pow(x, 3)*pow(y, 2) - 5*pow(x, 3)*pow(z, 2) + (25.0/16.0)*x*pow(y, 4) - 15*x*pow(y, 2)*pow(z, 2) + 5*x*pow(z, 4));
        B[2] += G * (-10*pow(x, 3)*y*z - 10*x*pow(y, 3)*z + 20*x*y*pow(z, 3));
        if (dB) {
            dB[0][0] += G * ((25.0/4.0)*pow(x, 3)*y + (15.0/4.0)*x*pow(y, 3) - 30*x*y*pow(z, 2));
            dB[0][1] += G * ((25.0/16.0)*pow(x, 4) + (45.0/8.0)*pow(x, 2)*pow(y, 2) - 15*pow(x, 2)*pow(z, 2) + (25.0/16.0)*pow(y, 4) - 15*pow(y, 2)*pow(z, 2) + 5*pow(z, 4));
            dB[0][2] += G * (-30*pow(x, 2)*y*z - 10*pow(y, 3)*z + 20*y*pow(z, 3));
            dB[1][0] += G * ((25.0/16.0)*pow(x, 4) + (45.0/8.0)*pow(x, 2)*pow(y, 2) - 15*pow(x, 2)*pow(z, 2) + (25.0/16.0)*pow(y, 4) - 15*pow(y, 2)*pow(z, 2) + 5*pow(z, 4));
            dB[1][1] += G * ((15.0/4.0)*pow(x, 3)*y + (25.0/4.0)*x*pow(y, 3) - 30*x*y*pow(z, 2));
            dB[1][2] += G * (-10*pow(x, 3)*z - 30*x*pow(y, 2)*z + 20*x*pow(z, 3));
            dB[2][0] += G * (-30*pow(x, 2)*y*z - 10*pow(y, 3)*z + 20*y*pow(z, 3));
            dB[2][1] += G * (-10*pow(x, 3)*z - 30*x*pow(y, 2)*z + 20*x*pow(z, 3));
            dB[2][2] += G * (-10*pow(x, 3)*y - 10*x*pow(y, 3) + 60*x*y*pow(z, 2));
        }
        return true;
    }
    if (l == 5 && m == -1) {
        B[0] += G * ((5.0/2.0)*pow(x, 3)*y*z + (5.0/2.0)*x*pow(y, 3)*z - 5*x*y*pow(z, 3));
        B[1] += G * ((5.0/8.0)*pow(x, 4)*z + (15.0/4.0)*pow(x, 2)*pow(y, 2)*z - 5.0/2.0*pow(x, 2)*pow(z, 3) + (25.0/8.0)*pow(y, 4)*z - 15.0/2.0*pow(y, 2)*pow(z, 3) + pow(z, 5));
        B[2] += G * ((5.0/8.0)*pow(x, 4)*y + (5.0/4.0)*pow(x, 2)*pow(y, 3) - 15.0/2.0*pow(x, 2)*y*pow(z, 2) + (5.0/8.0)*pow(y, 5) - 15.0/2.0*pow(y, 3)*pow(z, 2) + 5*y*pow(z, 4));
        if (dB) {
            dB[0][0] += G * ((15.0/2.0)*pow(x, 2)*y*z + (5.0/2.0)*pow(y, 3)*z - 5*y*pow(z, 3));
            dB[0][1] += G * ((5.0/2.0)*pow(x, 3)*z + (15.0/2.0)*x*pow(y, 2)*z - 5*x*pow(z, 3));
            dB[0][2] += G * ((5.0/2.0)*pow(x, 3)*y + (5.0/2.0)*x*pow(y, 3) - 15*x*y*pow(z, 2));
            dB[1][0] += G * ((5.0/2.0)*pow(x, 3)*z + (15.0/2.0)*x*pow(y, 2)*z - 5*x*pow(z, 3));
            dB[1][1] += G * ((15.0/2.0)*pow(x, 2)*y*z + (25.0/2.0)*pow(y, 3)*z - 15*y*pow(z, 3));
            dB[1][2] += G * ((5.0/8.0)*pow(x, 4) + (15.0/4.0)*pow(x, 2)*pow(y, 2) - 15.0/2.0*pow(x, 2)*pow(z, 2) + (25.0/8.0)*pow(y, 4) - 45.0/2.0*pow(y, 2)*pow(z, 2) + 5*pow(z, 4));
            dB[2][0] += G * ((5.0/2.0)*pow(x, 3)*y + (5.0/2.0)*x*pow(y, 3) - 15*x*y*pow(z, 2));
            dB[2][1] += G * ((5.0/8.0)*pow(x, 4) + (15.0/4.0)*pow(x, 2)*pow(y, 2) - 15.0/2.0*pow(x, 2)*pow(z, 2) + (25.0/8.0)*pow(y, 4) - 45.0/2.0*pow(y, 2)*pow(z, 2) + 5*pow(z, 4));
            dB[2][2] += G * (-15*pow(x, 2)*y*z - 15*pow(y, 3)*z + 20*y*pow(z, 3));
        }
        return true;
    }
    if (l == 5 && m == 0) {
        B[0] += G * (-5.0/16.0*pow(x, 5) - 5.0/8.0*pow(x, 3)*pow(y, 2) + (15.0/4.0)*pow(x, 3)*pow(z, 2) - 5.0/16.0*x*pow(y, 4) + (15.0/4.0)*x*pow(y, 2)*pow(z, 2) - 5.0/2.0*x*pow(z, 4));
        B[1] += G * (-5.0/16.0*pow(x, 4)*y - 5.0/8.0*pow(x, 2)*pow(y, 3) + (15.0/4.0)*pow(x, 2)*y*pow(z, 2) - 5.0/16.0*pow(y, 5) + (15.0/4.0)*pow(y, 3)*pow(z, 2) - 5.0/2.0*y*pow(z, 4));
        B[2] += G * ((15.0/8.0)*pow(x, 4)*z + (15.0/4.0)*pow(x, 2)*pow(y, 2)*z - 5*pow(x, 2)*pow(z, 3) + (15.0/8.0)*pow(y, 4)*z - 5*pow(y, 2)*pow(z, 3) + pow(z, 5));
        if (dB) {
            dB[0][0] += G * (-25.0/16.0*pow(x, 4) - 15.0/8.0*pow(x, 2)*pow(y, 2) + (45.0/4.0)*pow(x, 2)*pow(z, 2) - 5.0/16.0*pow(y, 4) + (15.0/4.0)*pow(y, 2)*pow(z, 2) - 5.0/2.0*pow(z, 4));
            dB[0][1] += G * (-5.0/4.0*pow(x, 3)*y - 5.0/4.0*x*pow(y, 3) + (15.0/2.0)*x*y*pow(z, 2));
            dB[0][2] += G * ((15.0/2.0)*pow(x, 3)*z + (15.0/2.0)*x*pow(y, 2)*z - 10*x*pow(z, 3));
            dB[1][0] += G * (-5.0/4.0*pow(x, 3)*y - 5.0/4.0*x*pow(y, 3) + (15.0/2.0)*x*y*pow(z, 2));
            dB[1][1] += G * (-5.0/16.0*pow(x, 4) - 15.0/8.0*pow(x, 2)*pow(y, 2) + (15.0/4.0)*pow(x, 2)*pow(z, 2) - 25.0/16.0*pow(y, 4) + (45.0/4.0)*pow(y, 2)*pow(z, 2) - 5.0/2.0*pow(z, 4));
            dB[1][2] += G * ((15.0/2.0)*pow(x, 2)*y*z + (15.0/2.0)*pow(y, 3)*z - 10*y*pow(z, 3));
            dB[2][0] += G * ((15.0/2.0)*pow(x, 3)*z + (15.0/2.0)*x*pow(y, 2)*z - 10*x*pow(z, 3));
            dB[2][1] += G * ((15.0/2.0)*pow(x, 2)*y*z + (15.0/2.0)*pow(y, 3)*z - 10*y*pow(z, 3));
            dB[2][2] += G * ((15.0/8.0)*pow(x, 4) + (15.0/4.0)*pow(x, 2)*pow(y, 2) - 15*pow(x, 2)*pow(z, 2) + (15.0/8.0)*pow(y, 4) - 15*pow(y, 2)*pow(z, 2) + 5*pow(z, 4));
        }
        return true;
    }
    if (l == 5 && m == 1) {
        B[0] += G * ((25.0/8.0)*pow(x, 4)*z + (15.0/4.0)*pow(x, 2)*pow(y, 2)*z - 15.0/2.0*pow(x, 2)*pow(z, 3) + (5.0/8.0)*pow(y, 4)*z - 5.0/2.0*pow(y, 2)*pow(z, 3) + pow(z, 5));
        B[1] += G * ((5.0/2.0)*pow(x, 3)*y*z + (5.0/2.0)*x*pow(y, 3)*z - 5*x*y*pow(z, 3));
        B[2] += G * ((5.0/8.0)*pow(x, 5) + (5.0/4.0)*pow(x, 3)*pow(y, 2) - 15.0/2.0*pow(x, 3)*pow(z, 2) + (5.0/8.0)*x*pow(y, 4) - 15.0/2.0*x*pow(y, 2)*pow(z, 2) + 5*x*pow(z, 4));
        if (dB) {
            dB[0][0] += G * ((25.0/2.0)*pow(x, 3)*z + (15.0/2.0)*x*pow(y, 2)*z - 15*x*pow(z, 3));
            dB[0][1] += G * ((15.0/2.0)*pow(x, 2)*y*z + (5.0/2.0)*pow(y, 3)*z - 5*y*pow(z, 3));
            dB[0][2] += G * ((25.0/8.0)*pow(x, 4) + (15.0/4.0)*pow(x, 2)*pow(y, 2) - 45.0/2.0*pow(x, 2)*pow(z, 2) + (5.0/8.0)*pow(y, 4) - 15.0/2.0*pow(y, 2)*pow(z, 2) + 5*pow(z, 4));
            dB[1][0] += G * ((15.0/2.0)*pow(x, 2)*y*z + (5.0/2.0)*pow(y, 3)*z - 5*y*pow(z, 3));
            dB[1][1] += G * ((5.0/2.0)*pow(x, 3)*z + (15.0/2.0)*x*pow(y, 2)*z - 5*x*pow(z, 3));
            dB[1][2] += G * ((5.0/2.0)*pow(x, 3)*y + (5.0/2.0)*x*pow(y, 3) - 15*x*y*pow(z, 2));
            dB[2][0] += G * ((25.0/8.0)*pow(x, 4) + (15.0/4.0)*pow(x, 2)*pow(y, 2) - 45.0/2.0*pow(x, 2)*pow(z, 2) + (5.0/8.0)*pow(y, 4) - 15.0/2.0*pow(y, 2)*pow(z, 2) + 5*pow(z, 4));
            dB[2][1] += G * ((5.0/2.0)*pow(x, 3)*y + (5.0/2.0)*x*pow(y, 3) - 15*x*y*pow(z, 2));
            dB[2][2] += G * (-15*pow(x, 3)*z - 15*x*pow(y, 2)*z + 20*x*pow(z, 3));
        }
        return true;
    }
    if (l == 5 && m == 2) {
        B[0] += G * ((15.0/16.0)*pow(x, 5) + (5.0/8.0)*pow(x, 3)*pow(y, 2) - 10*pow(x, 3)*pow(z, 2) - 5.0/16.0*x*pow(y, 4) + 5*x*pow(z, 4));
        B[1] += G * ((5.0/16.0)*pow(x, 4)*y - 5.0/8.0*pow(x, 2)*pow(y, 3) - 15.0/16.0*pow(y, 5) + 10*pow(y, 3)*pow(z, 2) - 5*y*pow(z, 4));
        B[2] += G * (-5*pow(x, 4)*z + 10*pow(x, 2)*pow(z, 3) + 5*pow(y, 4)*z - 10*pow(y, 2)*pow(z, 3));
        if (dB) {
            dB[0][0] += G * ((75.0/16.0)*pow(x, 4) + (15.0/8.0)*pow(x, 2)*pow(y, 2) - 30*pow(x, 2)*pow(z, 2) - 5.0/16.0*pow(y, 4) + 5*pow(z, 4));
            dB[0][1] += G * ((5.0/4.0)*pow(x, 3)*y - 5.0/4.0*x*pow(y, 3));
            dB[0][2] += G * (-20*pow(x, 3)*z + 20*x*pow(z, 3));
            dB[1][0] += G * ((5.0/4.0)*pow(x, 3)*y - 5.0/4.0*x*pow(y, 3));
            dB[1][1] += G * ((5.0/16.0)*pow(x, 4) - 15.0/8.0*pow(x, 2)*pow(y, 2) - 75.0/16.0*pow(y, 4) + 30*pow(y, 2)*pow(z, 2) - 5*pow(z, 4));
            dB[1][2] += G * (20*pow(y, 3)*z - 20*y*pow(z, 3));
            dB[2][0] += G * (-20*pow(x, 3)*z + 20*x*pow(z, 3));
            dB[2][1] += G * (20*pow(y, 3)*z - 20*y*pow(z, 3));
            dB[2][2] += G * (-5*pow(x, 4) + 30*pow(x, 2)*pow(z, 2) + 5*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
        }
        return true;
    }
    if (l == 5 && m == 3) {
        B[0] += G * (-25.0/4.0*pow(x, 4)*z + (15.0/2.0)*pow(x, 2)*pow(y, 2)*z + 10*pow(x, 2)*pow(z, 3) + (15.0/4.0)*pow(y, 4)*z - 10*pow(y, 2)*pow(z, 3));
        B[1] += G * (5*pow(x, 3)*y*z + 15*x*pow(y, 3)*z - 20*x*y*pow(z, 3));
        B[2] += G * (-5.0/4.0*pow(x, 5) + (5.0/2.0)*pow(x, 3)*pow(y, 2) + 10*pow(x, 3)*pow(z, 2) + (15.0/4.0)*x*pow(y, 4) - 30*x*pow(y, 2)*pow(z, 2));
        if (dB) {
            dB[0][0] += G * (-25*pow(x, 3)*z + 15*x*pow(y, 2)*z + 20*x*pow(z, 3));
            dB[0][1] += G * (15*pow(x, 2)*y*z + 15*pow(y, 3)*z - 20*y*pow(z, 3));
            dB[0][2] += G * (-25.0/4.0*pow(x, 4) + (15.0/2.0)*pow(x, 2)*pow(y, 2) + 30*pow(x, 2)*pow(z, 2) + (15.0/4.0)*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
            dB[1][0] += G * (15*pow(x, 2)*y*z + 15*pow(y, 3)*z - 20*y*pow(z, 3));
            dB[1][1] += G * (5*pow(x, 3)*z + 45*x*pow(y, 2)*z - 20*x*pow(z, 3));
            dB[1][2] += G * (5*pow(x, 3)*y + 15*x*pow(y, 3) - 60*x*y*pow(z, 2));
            dB[2][0] += G * (-25.0/4.0*pow(x, 4) + (15.0/2.0)*pow(x, 2)*pow(y, 2) + 30*pow(x, 2)*pow(z, 2) + (15.0/4.0)*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
            dB[2][1] += G * (5*pow(x, 3)*y + 15*x*pow(y, 3) - 60*x*y*pow(z, 2));
            dB[2][2] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
        }
        return true;
    }
    if (l == 5 && m == 4) {
        B[0] += G * (-3.0/2.0*pow(x, 5) + 5*pow(x, 3)*pow(y, 2) + 10*pow(x, 3)*pow(z, 2) + (5.0/2.0)*x*pow(y, 4) - 30*x*pow(y, 2)*pow(z, 2));
        B[1] += G * ((5.0/2.0)*pow(x, 4)*y + 5*pow(x, 2)*pow(y, 3) - 30*pow(x, 2)*y*pow(z, 2) - 3.0/2.0*pow(y, 5) + 10*pow(y, 3)*pow(z, 2));
        B[2] += G * (5*pow(x, 4)*z - 30*pow(x, 2)*pow(y, 2)*z + 5*pow(y, 4)*z);
        if (dB) {
            dB[0][0] += G * (-15.0/2.0*pow(x, 4) + 15*pow(x, 2)*pow(y, 2) + 30*pow(x, 2)*pow(z, 2) + (5.0/2.0)*pow(y, 4) - 30*pow(y, 2)*pow(z, 2));
            dB[0][1] += G * (10*pow(x, 3)*y + 10*x*pow(y, 3) - 60*x*y*pow(z, 2));
            dB[0][2] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
            dB[1][0] += G * (10*pow(x, 3)*y + 10*x*pow(y, 3) - 60*x*y*pow(z, 2));
            dB[1][1] += G * ((5.0/2.0)*pow(x, 4) + 15*pow(x, 2)*pow(y, 2) - 30*pow(x, 2)*pow(z, 2) - 15.0/2.0*pow(y, 4) + 30*pow(y, 2)*pow(z, 2));
            dB[1][2] += G * (-60*pow(x, 2)*y*z + 20*pow(y, 3)*z);
            dB[2][0] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
            dB[2][1] += G * (-60*pow(x, 2)*y*z + 20*pow(y, 3)*z);
            dB[2][2] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
        }
        return true;
    }
    if (l == 5 && m == 5) {
        B[0] += G * (5*pow(x, 4)*z - 30*pow(x, 2)*pow(y, 2)*z + 5*pow(y, 4)*z);
        B[1] += G * (-20*pow(x, 3)*y*z + 20*x*pow(y, 3)*z);
        B[2] += G * (pow(x, 5) - 10*pow(x, 3)*pow(y, 2) + 5*x*pow(y, 4));
        if (dB) {
            dB[0][0] += G * (20*pow(x, 3)*z - 60*x*pow(y, 2)*z);
            dB[0][1] += G * (-60*pow(x, 2)*y*z + 20*pow(y, 3)*z);
            dB[0][2] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
            dB[1][0] += G * (-60*pow(x, 2)*y*z + 20*pow(y, 3)*z);
            dB[1][1] += G * (-20*pow(x, 3)*z + 60*x*pow(y, 2)*z);
            dB[1][2] += G * (-20*pow(x, 3)*y + 20*x*pow(y, 3));
            dB[2][0] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
            dB[2][1] += G * (-20*pow(x, 3)*y + 20*x*pow(y, 3));
        }
        return true;
    }
    if (l == 5 && m == 6) {
        B[0] += G * (pow(x, 5) - 10*pow(x, 3)*pow(y, 2) + 5*x*pow(y, 4));
        B[1] += G * (-5*pow(x, 4)*y + 10*pow(x, 2)*pow(y, 3) - pow(y, 5));
        B[2] += G * (0);
        if (dB) {
            dB[0][0] += G * (5*pow(x, 4) - 30*pow(x, 2)*pow(y, 2) + 5*pow(y, 4));
            dB[0][1] += G * (-20*pow(x, 3)*y + 20*x*pow(y, 3));
            dB[1][0] += G * (-20*pow(x, 3)*y + 20*x*pow(y, 3));
            dB[1][1] += G * (-5*pow(x, 4) + 30*pow(x, 2)*pow(y, 2) - 5*pow(y, 4));
        }
        return true;
    }
    (void)x; (void)y; (void)z;
    return false;
}

/*
 * pt_solenoid.h -- field of a finite ideal solenoid in closed form, shared by
 * the CUDA kernels and the CPU oracle (the reference has no solenoid field
 * type; its configurations approximate one with Conductor segments).
 *
 * The solenoid is a sheet current on the cylinder rho = a, |z| <= b about the
 * z axis.  With z+- = z +- b, B0 = mu0 n I / pi,
 *   alpha+- = a / sqrt(z+-^2 + (rho + a)^2),  beta+- = z+- alpha+- / a,
 *   gamma = (a - rho) / (a + rho),
 *   k+- = sqrt((z+-^2 + (a - rho)^2) / (z+-^2 + (a + rho)^2)),
 *   B_rho = B0 [alpha+ C(k+, 1, 1, -1) - alpha- C(k-, 1, 1, -1)],
 *   B_z   = B0 a / (a + rho) [beta+ C(k+, gamma^2, 1, gamma) - beta- C(k-, gamma^2, 1, gamma)]
 * (Derby and Olbert, "Cylindrical magnets and ideal solenoids", Am. J. Phys.
 * 78, 229 (2010)), where C(kc, p, c, s) is Bulirsch's generalised complete
 * elliptic integral, evaluated with his iteration (Bulirsch, "Numerical
 * calculation of elliptic integrals and elliptic functions III", Numer.
 * Math. 13, 305 (1969)).  The field at the centre is mu0 n I b / sqrt(a^2 + b^2),
 * so B0 = B_centre sqrt(a^2 + b^2) / (pi b).
 *
 * The Jacobian comes from central differences of (B_rho, B_z) in rho and z
 * (step 1e-6 a; relative error ~1e-10 for fields that vary on the scale a)
 * and the cylindrical-to-Cartesian chain rule.
 */
#ifndef PT_SOLENOID_H
#define PT_SOLENOID_H

#include <math.h>

#if defined(__CUDACC__)
#define PTS_FN __host__ __device__ __forceinline__
#else
#define PTS_FN static inline
#endif

/* Bulirsch's cel(kc, p, c, s) = int_0^{pi/2} (c cos^2 + s sin^2) /
 * ((cos^2 + p sin^2) sqrt(cos^2 + kc^2 sin^2)) dphi, kc != 0 */
PTS_FN double pts_cel(double kc, double p, double c, double s) {
    const double errtol = 1e-15;
    double k = fabs(kc), pp = p, cc = c, ss = s, em = 1.0;
    if (p > 0) {
        pp = sqrt(p);
        ss = s / pp;
    } else {
        double f = kc * kc, q = 1.0 - f, g = 1.0 - pp;
        f = f - pp;
        q = q * (ss - c * pp);
        pp = sqrt(f / g);
        cc = (c - ss) / g;
        ss = -q / (g * g * pp) + cc * pp;
    }
    double f = cc;
    cc = cc + ss / pp;
    double g = k / pp;
    ss = 2.0 * (ss + f * g);
    pp = g + pp;
    g = em;
    em = k + em;
    double kk = k;
    for (int it = 0; it < 64 && fabs(g - k) > g * errtol; ++it) {
        k = 2.0 * sqrt(kk);
        kk = k * em;
        f = cc;
        cc = cc + ss / pp;
        g = kk / pp;
        ss = 2.0 * (ss + f * g);
        pp = g + pp;
        g = em;
        em = k + em;
    }
    return 1.5707963267948966 * (ss + cc * em) / (em * (em + pp));
}

/* (B_rho, B_z) at (rho >= 0, z) of the solenoid (radius a, half length b, B0 = mu0 n I / pi) */
PTS_FN void pts_solenoid_rz(double a, double b, double B0, double rho, double z, double *Br, double *Bz) {
    const double zp = z + b, zm = z - b;
    const double ap = a / sqrt(zp * zp + (rho + a) * (rho + a)), am = a / sqrt(zm * zm + (rho + a) * (rho + a));
    const double bp = zp * ap / a, bm = zm * am / a;
    const double gm = (a - rho) / (a + rho);
    const double kp = sqrt((zp * zp + (a - rho) * (a - rho)) / (zp * zp + (a + rho) * (a + rho)));
    const double km = sqrt((zm * zm + (a - rho) * (a - rho)) / (zm * zm + (a + rho) * (a + rho)));
    *Br = B0 * (ap * pts_cel(kp, 1.0, 1.0, -1.0) - am * pts_cel(km, 1.0, 1.0, -1.0));
    *Bz = B0 * a / (a + rho) * (bp * pts_cel(kp, gm * gm, 1.0, gm) - bm * pts_cel(km, gm * gm, 1.0, gm));
}

/* Cartesian B (and dB[i][j] = dB_i/dx_j when dB != 0) at (X, Y, Z) relative to the centre */
PTS_FN void pts_solenoid_field(double a, double b, double B0, double X, double Y, double Z, double B[3], double (*dB)[3]) {
    const double rho = sqrt(X * X + Y * Y);
    double Br, Bz;
    pts_solenoid_rz(a, b, B0, rho, Z, &Br, &Bz);
    const double c = rho > 0 ? X / rho : 1.0, s = rho > 0 ? Y / rho : 0.0;
    B[0] = Br * c;
    B[1] = Br * s;
    B[2] = Bz;
    if (!dB) return;
    const double h = 1e-6 * a;
    double Brp, Bzp, Brm, Bzm;
    pts_solenoid_rz(a, b, B0, rho + h, Z, &Brp, &Bzp);
    pts_solenoid_rz(a, b, B0, fabs(rho - h), Z, &Brm, &Bzm);
    if (rho - h < 0) Brm = -Brm; /* B_rho is odd and B_z even in rho */
    const double dBr_dr = (Brp - Brm) / (2 * h), dBz_dr = (Bzp - Bzm) / (2 * h);
    pts_solenoid_rz(a, b, B0, rho, Z + h, &Brp, &Bzp);
    pts_solenoid_rz(a, b, B0, rho, Z - h, &Brm, &Bzm);
    const double dBr_dz = (Brp - Brm) / (2 * h), dBz_dz = (Bzp - Bzm) / (2 * h);
    const double q = rho > 1e-9 * a ? Br / rho : dBr_dr; /* B_rho / rho, its limit on the axis */
    dB[0][0] = dBr_dr * c * c + q * s * s;
    dB[0][1] = (dBr_dr - q) * c * s;
    dB[0][2] = dBr_dz * c;
    dB[1][0] = (dBr_dr - q) * c * s;
    dB[1][1] = dBr_dr * s * s + q * c * c;
    dB[1][2] = dBr_dz * s;
    dB[2][0] = dBz_dr * c;
    dB[2][1] = dBz_dr * s;
    dB[2][2] = dBz_dz;
}

#endif

/*
 * pt_mr.cuh -- MicroRoughness scattering of neutrons at walls
 * (src/microroughness.cpp:15-134, used by TNeutron::OnHit,
 * src/neutron.cpp:38-62, 118-148, 187-264).
 *
 * The model gives, per wall contact, the probability of a diffuse
 * reflection (transmission) as the integral of the scattering distribution
 * MRDist over the polar angle, and samples the outgoing direction from it by
 * rejection.  The reference integrates with Boost.odeint's integrate() (a
 * Dormand-Prince 5(4) dense-output stepper, absolute and relative tolerance
 * 1e-6, first step 0.01); this file restates that integration, and finds the
 * rejection envelope's maximum from a grid refined by golden-section search
 * where the reference runs ALGLIB's conjugate-gradient minimiser from pi/4
 * (a local search that can stop below the maximum and clip the sampled
 * distribution).  The complex
 * amplitudes are written in real arithmetic (their squared moduli are all
 * the distribution uses), and the phi-integrated Bessel factor I0 is a power
 * series (an asymptotic series above 500).  All of it runs only for
 * materials with a roughness and a correlation length, out of line.
 */
#pragma once
#include "pt_device.cuh"

namespace ptd {
namespace {

/* MRDist's inputs that do not depend on the outgoing direction */
struct MRHit {
    double E, Estep;   /* kinetic energy 0.5 m_n v^2 and potential step [eV] */
    double ki, kt;     /* wave numbers in the first and the second solid [1/m] (kt = 0 when E <= Estep) */
    double kc2;        /* square of the critical wave number (negative for Estep < 0) */
    double cti, sti;   /* cosine and sine of the incidence angle to the normal */
    double si2;        /* |S_i|^2, the specularly transmitted amplitude's squared modulus */
    double b, w;       /* RMS roughness, correlation length [m] */
};

/* MR::MRValid (src/microroughness.cpp:15-33) */
__device__ __forceinline__ bool mr_valid(const double v[3], double Estep, double b, double w) {
    if (b == 0 || w == 0) return false;
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double E = 0.5 * PT_M_N * v2;
    const double ki = sqrt(2 * PT_M_N * E) * PT_ELE_E / PT_HBAR;
    if (Estep >= 0) {
        const double kc = sqrt(2 * PT_M_N * Estep) * PT_ELE_E / PT_HBAR;
        return 2 * b * ki < 2 && 2 * b * kc < 2;
    }
    const double kt = sqrt(2 * PT_M_N * (E - Estep)) * PT_ELE_E / PT_HBAR;
    return 2 * b * ki < 2 && 2 * b * kt < 2;
}

/* 4 c^2 / |c + sqrt(d)|^2 for real c >= 0 and d: the squared modulus of
 * the amplitude 2c / (c + sqrt(d)) with the complex square root */
__device__ __forceinline__ double mr_amp2(double c, double d) {
    if (d >= 0) {
        const double s = c + sqrt(d);
        return 4 * c * c / (s * s);
    }
    return 4 * c * c / (c * c - d);
}

__device__ __noinline__ void mr_setup(MRHit &h, const double v[3], const double n[3], double Estep, double b, double w) {
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double vn = v[0] * n[0] + v[1] * n[1] + v[2] * n[2];
    h.E = 0.5 * PT_M_N * v2;
    h.Estep = Estep;
    h.ki = sqrt(2 * PT_M_N * h.E) * PT_ELE_E / PT_HBAR;
    const double kc = sqrt(2 * PT_M_N * fabs(Estep)) * PT_ELE_E / PT_HBAR;
    h.kc2 = Estep >= 0 ? kc * kc : -(kc * kc);
    h.kt = h.E > Estep ? sqrt(2 * PT_M_N * (h.E - Estep)) * PT_ELE_E / PT_HBAR : 0.0;
    h.cti = fabs(vn / sqrt(v2));
    h.sti = sin(acos(h.cti));
    h.si2 = mr_amp2(h.cti, h.cti * h.cti - h.kc2 / h.ki / h.ki);
    h.b = b;
    h.w = w;
}

/* exp(-a) * 2 pi I0(x) for a >= x >= 0 (I0: modified Bessel function of the
 * first kind, order 0) */
__device__ __forceinline__ double mr_exp_i0(double a, double x) {
    if (x <= 500.0) {
        const double q = 0.25 * x * x;
        double term = 1.0, sum = 1.0;
        for (int k = 1; k < 2000; ++k) {
            term = term * q / ((double)k * (double)k);
            sum += term;
            if (term < 1e-17 * sum) break;
        }
        return exp(-a) * 2 * PT_PI * sum;
    }
    /* e^-x I0(x) ~ (2 pi x)^-1/2 sum_k ((2k-1)!!)^2 / (k! (8x)^k) */
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 12; ++k) {
        term = term * (2.0 * k - 1) * (2.0 * k - 1) / ((double)k * 8.0 * x);
        sum += term;
    }
    return exp(x - a) * 2 * PT_PI * sum / sqrt(2 * PT_PI * x);
}

/* MR::MRDist (src/microroughness.cpp:35-85): the scattering distribution at
 * polar angle theta and azimuth phi; `integral`: integrated over phi and
 * times sin(theta) */
__device__ __noinline__ double mr_dist(const MRHit &h, bool transmit, bool integral, double theta, double phi) {
    if (theta < 0 || theta > PT_PI / 2) return 0;
    if (transmit && h.E <= h.Estep) return 0;
    const double ct = cos(theta), st = sin(theta);
    double so2;
    if (transmit) {
        if (-h.kc2 / h.kt / h.kt > ct * ct) return 0;
        so2 = mr_amp2(ct, ct * ct + h.kc2 / h.kt / h.kt);
    } else {
        so2 = mr_amp2(ct, ct * ct - h.kc2 / h.ki / h.ki);
    }
    const double b = h.b, w = h.w, ki = h.ki, kt = h.kt, sti = h.sti;
    double Fmu;
    if (!integral && !transmit)
        Fmu = exp(-w * w / 2 * ki * ki * (sti * sti + st * st - 2 * sti * st * cos(phi)));
    else if (!integral && transmit)
        Fmu = exp(-w * w / 2 * (ki * ki * sti * sti + kt * kt * st * st - 2 * ki * kt * sti * st * cos(phi)));
    else if (!transmit)
        Fmu = mr_exp_i0(w * w / 2 * ki * ki * (sti * sti + st * st), w * w * ki * ki * sti * st);
    else
        Fmu = mr_exp_i0(w * w / 2 * (ki * ki * sti * sti + kt * kt * st * st), w * w * ki * kt * sti * st);
    double factor = h.kc2 * h.kc2 * b * b * w * w / 8 / PT_PI / h.cti;
    if (transmit) factor *= kt / ki;
    if (integral) factor *= st;
    return factor * h.si2 * so2 * Fmu;
}

/* MR::MRProb (src/microroughness.cpp:101-107): the integral of the
 * phi-integrated distribution over theta in [0, pi/2] as odeint's
 * integrate() computes it -- Dormand-Prince 5(4) with its dense-output
 * controller (error max |err| / (1e-6 + 1e-6 (|x| + dt |dx/dt|)); a
 * rejected step shrinks by max(0.9 err^-1/3, 0.2), an accepted one with
 * err < 0.5 grows by 0.9 max(err, 5^-5)^-1/5), first step 0.01, and the
 * last step shortened to end at pi/2.  `ok` turns false after 500
 * rejected tries of one step or 100,000 steps. */
__device__ __noinline__ double mr_prob(const MRHit &h, bool transmit, bool &ok) {
    const double T = PT_PI / 2;
    double t = 0.0, x = 0.0, dt = 0.01;
    double k1 = mr_dist(h, transmit, true, t, 0.0);
    int steps = 0;
    while (T - t > 2.220446049250313e-16) {
        while (t + dt - T <= 2.220446049250313e-16) {
            int tries = 0;
            for (;;) {
                /* the integrand does not depend on x, so the second stage (weight 0 in
                 * both solutions) is not needed */
                const double k3 = mr_dist(h, transmit, true, t + dt * (3.0 / 10), 0.0);
                const double k4 = mr_dist(h, transmit, true, t + dt * (4.0 / 5), 0.0);
                const double k5 = mr_dist(h, transmit, true, t + dt * (8.0 / 9), 0.0);
                const double k6 = mr_dist(h, transmit, true, t + dt, 0.0);
                const double xn = x + dt * ((35.0 / 384) * k1 + (500.0 / 1113) * k3 + (125.0 / 192) * k4 +
                                            (-2187.0 / 6784) * k5 + (11.0 / 84) * k6);
                const double k7 = k6; /* the derivative at the new point: the integrand does not depend on x */
                const double xe = dt * ((35.0 / 384 - 5179.0 / 57600) * k1 + (500.0 / 1113 - 7571.0 / 16695) * k3 +
                                        (125.0 / 192 - 393.0 / 640) * k4 + (-2187.0 / 6784 + 92097.0 / 339200) * k5 +
                                        (11.0 / 84 - 187.0 / 2100) * k6 + (-1.0 / 40) * k7);
                double err = fabs(xe) / (1e-6 + 1e-6 * (fabs(x) + fabs(dt) * fabs(k1)));
                if (!(err <= 1.0)) {
                    if (!(err == err)) err = 1e300;
                    dt *= fmax(0.9 * pow(err, -1.0 / 3.0), 0.2);
                    if (++tries >= 500) { ok = false; return x; }
                    continue;
                }
                t += dt;
                x = xn;
                k1 = k7;
                if (err < 0.5) {
                    err = fmax(3.2e-4, err); /* 5^-5 */
                    dt *= 0.9 * pow(err, -1.0 / 5.0);
                }
                break;
            }
            if (++steps > 100000) { ok = false; return x; }
        }
        if (T - t > 2.220446049250313e-16) {
            dt = T - t;
            k1 = mr_dist(h, transmit, true, t, 0.0);
        }
    }
    return x;
}

/* MR::MRDistMax (src/microroughness.cpp:123-132): the largest of 65 grid
 * values of the distribution at phi = 0 over [0, pi/2], refined by 60
 * golden-section steps between the best point's neighbours, and of the
 * values beside the amplitude's cusp */
__device__ __noinline__ double mr_distmax(const MRHit &h, bool transmit) {
    const double step = PT_PI / 2 / 64;
    int best = 0;
    double fbest = mr_dist(h, transmit, false, 0.0, 0.0);
    for (int k = 1; k <= 64; ++k) {
        const double fk = mr_dist(h, transmit, false, k * step, 0.0);
        if (fk > fbest) { fbest = fk; best = k; }
    }
    const double g = 0.6180339887498949;
    double a = (best > 0 ? best - 1 : 0) * step, b = (best < 64 ? best + 1 : 64) * step;
    double c = b - g * (b - a), d = a + g * (b - a);
    double fc = mr_dist(h, transmit, false, c, 0.0), fd = mr_dist(h, transmit, false, d, 0.0);
    for (int i = 0; i < 60; ++i) {
        if (fc >= fd) {
            b = d; d = c; fd = fc;
            c = b - g * (b - a);
            fc = mr_dist(h, transmit, false, c, 0.0);
        } else {
            a = c; c = d; fc = fd;
            d = a + g * (b - a);
            fd = mr_dist(h, transmit, false, d, 0.0);
        }
    }
    double m = fmax(fbest, mr_dist(h, transmit, false, 0.5 * (a + b), 0.0));
    /* the cusp where the outgoing amplitude's square root turns complex
     * (reflection: cos theta = kc / ki above the step; transmission below a
     * negative step: the cut-off cos^2 theta = -kc^2 / kt^2, approached from
     * inside) is a local maximum narrower than the grid */
    double c2 = -1;
    if (!transmit && h.kc2 > 0 && h.kc2 < h.ki * h.ki) c2 = h.kc2 / (h.ki * h.ki);
    if (transmit && h.E > h.Estep && h.kc2 < 0 && -h.kc2 < h.kt * h.kt) c2 = -h.kc2 / (h.kt * h.kt);
    if (c2 > 0) {
        const double th = acos(sqrt(c2));
        const double fac[4] = {1 - 1e-12, 1 - 1e-9, 1 + 1e-12, 1 + 1e-9};
        for (int k = 0; k < 4; ++k) m = fmax(m, mr_dist(h, transmit, false, th * fac[k], 0.0));
    }
    return m;
}

} // namespace
} // namespace ptd
